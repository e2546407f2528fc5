"""Build libvegasgb.so (the CUDA kernels + C-ABI) for sm_103a with nvcc.

    python -m vegasflow_gb300.build [--force] [-v]

Each ``csrc/*.cu`` / ``*.cpp`` is compiled in parallel to an object file under
``vegasflow_gb300/_build/``, then linked into ``_build/libvegasgb.so``.  Objects
are rebuilt when any source or header is newer.  No CMake, one -gencode.
"""

from __future__ import annotations

import argparse
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libvegasgb.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              f"-I{INCLUDE}", f"-I{CSRC}", f"-I{BUILD}"]


def nvcc_path():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build vegasflow_gb300")


def cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc_path())))


# Sources compiled more than once, with per-variant defines (instantiation
# units split by block size and dimension range so they build in parallel).
VARIANTS = {
    "vf_vegas_f32_inst.cu": [
        (f"t{t}_{lo}_{hi}", [f"-DVF_INST_THREADS={t}", f"-DVF_INST_DLO={lo}", f"-DVF_INST_DHI={hi}"])
        for t, lo, hi in ((1024, 1, 4), (1024, 5, 8), (1024, 9, 12), (1024, 13, 16), (512, 1, 8), (512, 9, 16))],
    "vf_vegas_f32_inj.cu": [
        (f"d{lo}_{hi}", [f"-DVF_INST_DLO={lo}", f"-DVF_INST_DHI={hi}"]) for lo, hi in ((1, 8), (9, 16))],
}


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _units():
    """(source, object, extra flags) for every object of the library."""
    out = []
    for s in _sources():
        stem = os.path.splitext(os.path.basename(s))[0]
        for tag, flags in VARIANTS.get(os.path.basename(s), [(None, [])]):
            name = f"{stem}_{tag}" if tag else stem
            out.append((s, os.path.join(BUILD, name + ".o"), flags))
    return out


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
            + glob.glob(os.path.join(INCLUDE, "*.h")))


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _compile(src, obj, verbose, extra):
    cmd = [nvcc_path(), *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "cu"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)
    return obj


JIT_HEADERS = ("vf_device.cuh", "vf_sample.cuh", "vf_vegas_f32.cuh", "vf_plus_args.cuh", "vf_plus_sampler.cuh",
               "vf_plus_f32.cuh", "vf_batch_sampler.cuh")


def write_jit_sources():
    """Embed the sampler headers as strings for NVRTC (``_build/vf_jit_sources.h``)."""
    out = os.path.join(BUILD, "vf_jit_sources.h")
    parts = ["// Generated by vegasflow_gb300/build.py: the sampler headers for NVRTC.", "#pragma once",
             f"static const int kJitHeaderCount = {len(JIT_HEADERS)};",
             "static const char* kJitHeaderNames[] = {" + ", ".join(f'"{h}"' for h in JIT_HEADERS) + "};",
             "static const char* kJitHeaderSources[] = {"]
    for h in JIT_HEADERS:
        text = open(os.path.join(CSRC, h)).read()
        assert ")VFJIT\"" not in text
        parts.append('R"VFJIT(' + text + ')VFJIT",')
    parts.append("};")
    new = "\n".join(parts) + "\n"
    if not os.path.exists(out) or open(out).read() != new:
        with open(out, "w") as f:
            f.write(new)
    return out


def build(force=False, verbose=False, jobs=None, extra_flags=()):
    """Compile and link libvegasgb.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    write_jit_sources()
    hdr_time = _newest(_headers())
    todo = []
    objs = []  # only the current units' objects are linked (stale ones are ignored)
    for s, obj, flags in _units():
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(s), hdr_time):
            todo.append((s, obj, flags))
    jobs = jobs or min(len(todo) or 1, os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(lambda t: _compile(t[0], t[1], verbose, list(t[2]) + list(extra_flags)), todo))
    if force or todo or not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        home = cuda_home()
        lib64 = os.path.join(home, "lib64")
        cmd = [nvcc_path(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs,
               f"-L{lib64}", "-lcudart", "-lnvrtc", "-Xlinker", f"-rpath={lib64}"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    return LIB


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true", help="print -Xptxas -v register/smem usage")
    args = ap.parse_args(argv)
    extra = ["-Xptxas", "-v"] if args.ptxas_info else []
    path = build(force=args.force or args.ptxas_info, verbose=args.verbose or args.ptxas_info,
                 extra_flags=extra)
    print(path)


if __name__ == "__main__":
    sys.exit(main())
