// Host stand-in header for building the reference renderer on the CPU (test infrastructure).
#pragma once
#include "illume_ref_shim.h"
