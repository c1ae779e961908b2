"""Stage the MPT headers the reference-built checker needs -- TEST
INFRASTRUCTURE ONLY.

    python -m oracle.ref.stage [REFERENCE_SRC]

REFERENCE_SRC is the reference's src/ directory (default: the environment's
MPT_REFERENCE_SRC, else /root/reference/src, where the build container mounts
it).  The headers that oracle/ref/ref_driver.cpp and the nigh-adapter program
(tests/cpp/nigh_adapter.cpp) include, as g++ -MM lists them, are copied
unmodified into oracle/_ref/src/mpt/...  oracle/_ref is git-ignored: the copy
is a build input of the checker (compiled into oracle/_ref/libref.so where the
checker runs, including hosts that have no reference tree), never part of the
repository.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
STAGED = os.path.join(ORACLE, "_ref", "src")
DEFAULT_SOURCE = "/root/reference/src"

# the programs whose reference includes are staged
PROGRAMS = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(ROOT, "tests", "cpp", "nigh_adapter.cpp")]


def _deps(src_root: str, program: str):
    cmd = ["g++", "-std=c++17", "-fopenmp", "-DNDEBUG", "-DMPT_LOG_LEVEL=WARN", "-MM", "-MT", "x",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(HERE, "shim"), "-I", src_root, program]
    out = subprocess.run(cmd, capture_output=True, text=True, check=True).stdout
    root = os.path.realpath(src_root) + os.sep
    for tok in out.replace("\\\n", " ").split():
        if tok.endswith(":"):
            continue
        p = os.path.realpath(tok)
        if p.startswith(root):
            yield os.path.relpath(p, root)


def stage(src_root: str | None = None) -> str | None:
    """Copy the needed headers from src_root into oracle/_ref/src; returns the
    staged directory, or None when src_root holds no MPT sources."""
    src_root = src_root or os.environ.get("MPT_REFERENCE_SRC") or DEFAULT_SOURCE
    if not os.path.isdir(os.path.join(src_root, "mpt")):
        return None
    rels = sorted({r for prog in PROGRAMS for r in _deps(src_root, prog)})
    for rel in rels:
        dst = os.path.join(STAGED, rel)
        src = os.path.join(src_root, rel)
        if os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(src):
            continue
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        shutil.copyfile(src, dst)
    with open(os.path.join(STAGED, "STAGED_FILES"), "w") as f:
        f.write("\n".join(rels) + "\n")
    return STAGED


if __name__ == "__main__":
    d = stage(sys.argv[1] if len(sys.argv) > 1 else None)
    print(d or "no reference sources found")
