"""Builds libsandengine_gb300.so in-tree (sandengine_gb300/_build/).

The library holds the rule compiler (C++), the runtime and C ABI (C++), the
rule-set-independent device kernels (nvcc, sm_103a) and, as embedded source text, the
Margolus kernel template that NVRTC compiles together with each rule set's generated
code.  Translation units compile in parallel; no cmake.

    python -m sandengine_gb300.build        # or sandengine_gb300.build.build()
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsandengine_gb300.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HOST_SOURCES = ["lang/yaml.cpp", "lang/lang.cpp", "lang/codegen.cpp", "runtime/jit.cpp",
                "runtime/engine.cpp", "runtime/batch.cpp", "runtime/server.cpp", "runtime/snapshot.cpp",
                "capi.cpp"]
CUDA_SOURCES = ["kernels/devutil.cu", "kernels/render.cu"]
EMBED = [("SE_PRELUDE_SRC", "kernels/prelude.cuh"), ("SE_MARGOLUS_SRC", "kernels/margolus.cuh")]


def _embed_header() -> str:
    parts = ["// Generated by sandengine_gb300/build.py: kernel template sources for NVRTC.\n"]
    for name, rel in EMBED:
        with open(os.path.join(CSRC, rel)) as f:
            text = f.read()
        assert ")SEK\"" not in text
        parts.append(f'static const char* {name} = R"SEK({text})SEK";\n')
    return "".join(parts)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _all_inputs():
    files = []
    for root, _, names in os.walk(CSRC):
        for n in sorted(names):
            if n.endswith((".cpp", ".hpp", ".cu", ".cuh", ".h")):
                files.append(os.path.join(root, n))
    files.append(os.path.join(HERE, "..", "include", "sandengine.h"))
    files.append(os.path.abspath(__file__))
    return sorted(files)


def _fingerprint() -> str:
    h = hashlib.sha256()
    for p in _all_inputs():
        with open(p, "rb") as f:
            h.update(p.encode())
            h.update(f.read())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    stamp = os.path.join(OUT, "stamp")
    fp = _fingerprint()
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == fp:
        return LIB
    inc = os.path.join(OUT, "kernel_src.inc")
    with open(inc, "w") as f:
        f.write(_embed_header())
    common = ["-O2", "-std=c++20", "-Xcompiler", "-fPIC,-fvisibility=hidden", "-I", OUT, "-I", CSRC,
              "-I", os.path.join(HERE, "..", "include")]
    jobs = []
    for rel in HOST_SOURCES:
        obj = os.path.join(OUT, rel.replace("/", "_") + ".o")
        jobs.append([NVCC, *common, "-x", "c++", "-c", os.path.join(CSRC, rel), "-o", obj])
    for rel in CUDA_SOURCES:
        obj = os.path.join(OUT, rel.replace("/", "_") + ".o")
        jobs.append([NVCC, *common, *ARCH, "-lineinfo", "-c", os.path.join(CSRC, rel), "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(_run, jobs))
    objs = [j[-1] for j in jobs]
    tmp = LIB + f".tmp{os.getpid()}"
    _run([NVCC, "-shared", *ARCH, "-cudart", "static", *objs, "-o", tmp,
          "-L", os.path.join(CUDA_HOME, "lib64"), "-lnvrtc",
          "-Xlinker", "-rpath," + os.path.join(CUDA_HOME, "lib64")])
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(fp)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
