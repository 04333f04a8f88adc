"""In-tree build of the bicos_gb300 shared library for sm_103a.

Compiles every translation unit under csrc/ with nvcc in parallel (one
-gencode, sm_103a) and links ``libbicos_gb300/_lib/libbicos_gb300.so``.
No CMake, no torch extension machinery: the library exports a plain C ABI
(include/bicos_c.h) plus the C++ BICOS::match API (include/BICOS/).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libbicos_gb300.so")
GEN_DIR = os.path.join(OUT_DIR, "gen")
# trained weights of the learned subpixel proposal, compiled into the library
MODEL = os.path.join(PKG, "learned_subpixel.bsm")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def model_blob() -> str:
    """C++ source holding the model file's bytes (empty when there is no
    model file); rewritten only when its content changes."""
    data = open(MODEL, "rb").read() if os.path.exists(MODEL) else b""
    body = ",".join(str(b) for b in data) or "0"
    text = ("// generated by libbicos_gb300/build.py from learned_subpixel.bsm\n"
            "namespace bicos_gb300 {\n"
            f"extern const unsigned char kEmbeddedModel[] = {{{body}}};\n"
            f"extern const unsigned long long kEmbeddedModelSize = {len(data)}ull;\n"
            "}\n")
    os.makedirs(GEN_DIR, exist_ok=True)
    path = os.path.join(GEN_DIR, "learned_model_blob.cpp")
    if not os.path.exists(path) or open(path).read() != text:
        with open(path, "w") as f:
            f.write(text)
    return path


def _deps_newer(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    heads = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    inc = os.path.join(ROOT, "include")
    for dp, _, fs in os.walk(inc):
        heads += [os.path.join(dp, f) for f in fs]
    return any(os.path.getmtime(p) > t for p in [src] + heads)


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
    if _deps_newer(obj, src):
        cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc(), "-x", "cu"] + cmd[1:]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sources() + [model_blob()]
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra or []), srcs))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
