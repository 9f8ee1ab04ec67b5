// Definitions of the opaque C-ABI handles (include/illume.h).
#pragma once

#include "renderer.h"
#include "runtime.h"
#include "server.h"

struct illume_context { illume::Context c; };
struct illume_scene { illume::Scene s; };
struct illume_renderer { illume::Renderer r; };
struct illume_server { illume::Server s; };
