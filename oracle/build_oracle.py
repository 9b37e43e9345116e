"""Build recipe for the CPU oracle (test infrastructure only).

* ``build_oracle()`` compiles this project's C restatement ``oracle/sdf_oracle.c`` into
  ``oracle/_build/liboracle.so``. It runs on every machine that runs the tests.
* ``build_ref()`` compiles the reference's own CPU sources for the bake path -- the
  triangle/box test header, ``voxelize.cpp``, ``mesh_weld.cpp`` and ``mesh_validate.cpp`` --
  where they lie in the reference tree, against the small glm stand-in in
  ``oracle/glm_shim``, together with ``oracle/ref_driver.cpp``, into
  ``oracle/_ref/libitaly_ref.so``. It needs the reference tree: ``ITALY_REF_ROOT`` names it, else
  a ``reference`` folder beside this repository's root is used; without either the step is
  skipped (the prebuilt library, if any, is kept).

Both use ``-ffp-contract=off``: FP32 occupancy must round exactly as the reference does.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "liboracle.so")
REF_SO = os.path.join(REF_DIR, "libitaly_ref.so")
REF_ROOT = os.environ.get("ITALY_REF_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")

REF_SOURCES = [
    "src/convert/voxelize.cpp",
    "src/io/mesh_weld.cpp",
    "src/io/mesh_validate.cpp",
]


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources if os.path.exists(s))


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "sdf_oracle.c")
    if force or _stale(ORACLE_SO, [src, __file__]):
        os.makedirs(BUILD_DIR, exist_ok=True)
        tmp = ORACLE_SO + f".tmp{os.getpid()}"
        cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
               "-pthread", src, "-o", tmp, "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def ref_available() -> bool:
    return all(os.path.exists(os.path.join(REF_ROOT, s)) for s in REF_SOURCES) and os.path.exists(
        os.path.join(REF_ROOT, "src/convert/tri_box_overlap.h"))


def build_ref(force: bool = False) -> str | None:
    """Compile the reference's CPU bake-path sources; returns the .so path or None."""
    if not ref_available():
        return REF_SO if os.path.exists(REF_SO) else None
    srcs = [os.path.join(REF_ROOT, s) for s in REF_SOURCES]
    deps = srcs + [os.path.join(HERE, "ref_driver.cpp"), os.path.join(HERE, "glm_shim", "glm", "glm.hpp"),
                   os.path.join(REF_ROOT, "src/convert/tri_box_overlap.h"), __file__]
    if force or _stale(REF_SO, deps):
        os.makedirs(REF_DIR, exist_ok=True)
        tmp = REF_SO + f".tmp{os.getpid()}"
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
               "-I", os.path.join(HERE, "glm_shim"), "-I", os.path.join(REF_ROOT, "src"),
               os.path.join(HERE, "ref_driver.cpp"), *srcs, "-o", tmp]
        subprocess.run(cmd, check=True)
        os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
