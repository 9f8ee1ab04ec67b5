"""Build recipe for the reference renderer's own sources on the host (oracle/_ref/).

TEST INFRASTRUCTURE. Compiles the reference's src/ files where they lie (read-only), as
one g++ translation unit through oracle/ref_driver.cpp with the host shim headers of
oracle/ref_shim/, into oracle/_ref/libillume_ref.so. The library pins the oracle and
generates the golden fixtures of tests/golden/. Outputs go only into oracle/_ref/.

Only possible where the reference checkout exists: its root is read from the
environment variable ILLUME_REFERENCE_ROOT, else the build container's checkout path.
Returns None when there is no checkout there.

stage() copies the checkout's src/ and include/ (the files this build reads) into
oracle/_ref/reference/, which git ignores and which travels with the working tree to
the machines that have no checkout; there build(staged=True) compiles the same library
from that copy, for the bench's reference arm (the reference's own integrator timed on
that machine's host cores). Nothing else builds from the copy.

Scenes are loaded from a scratch copy of the needed OBJ files under oracle/_ref/work,
because the reference writes a BVH cache file next to every OBJ it loads
(src/primitives/mesh.cu:407-414, src/accel/bvh.cpp:399-417).
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("ILLUME_REFERENCE_ROOT", "/root/reference")
OUT_DIR = os.path.join(HERE, "_ref")
LIB_PATH = os.path.join(OUT_DIR, "libillume_ref.so")
WORK_DIR = os.path.join(OUT_DIR, "work")
STAGED_ROOT = os.path.join(OUT_DIR, "reference")


def available() -> bool:
    return os.path.isdir(os.path.join(REF_ROOT, "src"))


def staged_available() -> bool:
    return os.path.isdir(os.path.join(STAGED_ROOT, "src"))


def stage() -> bool:
    """Copy the checkout's src/ and include/ into oracle/_ref/reference/ (refreshed when
    the checkout's files are newer). Returns whether a copy is there."""
    if not available():
        return staged_available()
    for sub in ("src", "include"):
        src_dir = os.path.join(REF_ROOT, sub)
        for dirpath, _, files in os.walk(src_dir):
            rel = os.path.relpath(dirpath, REF_ROOT)
            os.makedirs(os.path.join(STAGED_ROOT, rel), exist_ok=True)
            for f in files:
                a, b = os.path.join(dirpath, f), os.path.join(STAGED_ROOT, rel, f)
                if not os.path.exists(b) or os.path.getmtime(a) > os.path.getmtime(b):
                    shutil.copy2(a, b)
    return True


def build(force: bool = False, staged: bool = False):
    """The library from the checkout, or with staged=True from the staged copy where
    there is no checkout; None when neither is there."""
    if available():
        root = REF_ROOT
    elif staged and staged_available():
        root = STAGED_ROOT
    else:
        return None
    os.makedirs(os.path.join(OUT_DIR, "inc"), exist_ok=True)
    # transform.h includes "rapidjson\document.h" (a Windows path): a file of that literal
    # name forwards to the real header.
    fwd = os.path.join(OUT_DIR, "inc", "rapidjson\\document.h")
    if not os.path.exists(fwd):
        with open(fwd, "w") as f:
            f.write('#include "rapidjson/document.h"\n')
    deps = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(HERE, "philox.h"),
            os.path.join(HERE, "ref_shim", "illume_ref_shim.h"), os.path.join(HERE, "..", "include", "illume.h")]
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(d) for d in deps):
        return LIB_PATH
    obj = os.path.join(OUT_DIR, "arraylist.o")
    subprocess.run(["gcc", "-O2", "-fPIC", "-c", os.path.join(root, "src", "arraylist.c"), "-o", obj], check=True)
    # -ftrivial-auto-var-init=zero gives the uninitialised AABB of get_bounds
    # (src/primitives/mesh.cu:345) a defined start value.
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-ftrivial-auto-var-init=zero", "-fPIC", "-shared", "-w",
           "-I", os.path.join(HERE, "ref_shim"), "-I", os.path.join(OUT_DIR, "inc"),
           "-I", os.path.join(root, "src"), "-I", os.path.join(root, "include"),
           os.path.join(HERE, "ref_driver.cpp"), obj, "-o", LIB_PATH]
    subprocess.run(cmd, check=True)
    return LIB_PATH


def prepare_work_dir(obj_files=("cube.obj", "quad.obj", "icosahedron.obj", "monkey.obj", "bunny5k.obj"),
                     scenes=("cornell_box.json", "cornell_spheres.json")) -> str:
    """Copy the OBJ assets and scene files the tests use into oracle/_ref/work."""
    os.makedirs(os.path.join(WORK_DIR, "res"), exist_ok=True)
    for o in obj_files:
        src = os.path.join(REF_ROOT, "res", o)
        dst = os.path.join(WORK_DIR, "res", o)
        if os.path.exists(src) and not os.path.exists(dst):
            shutil.copyfile(src, dst)
    for s in scenes:
        src = os.path.join(REF_ROOT, "res", "scenes", s)
        if os.path.exists(src):
            shutil.copyfile(src, os.path.join(WORK_DIR, s))
    return WORK_DIR


if __name__ == "__main__":
    print(build(force=True))
