"""Builds libsconegpu.so in-tree (scone_gb300/_build/) with nvcc for sm_103a.

Translation units compile in parallel.  The FP64 verification history loop and the support kernels
are compiled with -fmad=false (every multiply and add rounded separately, as SCONE's gfortran build
does on x86-64); the mixed-precision history loop keeps FMA contraction.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsconegpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-Xptxas", "-warn-spills"]
UNITS = {
    "sg_tr_fp64.cu": ["-fmad=false"],
    "sg_tr_mixed.cu": [],
    "sg_tr_ce_fp64.cu": ["-fmad=false"],
    "sg_tr_ce_mixed.cu": [],
    "sg_support.cu": ["-fmad=false"],
    "sg_host.cu": ["-fmad=false"],
    "sg_noalloc.cu": ["-fmad=false"],
    "sg_batch_fp64.cu": ["-fmad=false"],
    "sg_batch_mixed.cu": [],
    "sg_batch_host.cu": ["-fmad=false"],
}


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "scone_gpu.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in sources())


def build(force=False, verbose=False, extra=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    for unit, flags in UNITS.items():
        obj = os.path.join(OUT, unit.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *flags, *extra, "-c", os.path.join(CSRC, unit), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((unit, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    failed = []
    for unit, p in procs:
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        if p.returncode != 0:
            failed.append(unit)
            sys.stderr.write(text)
        elif verbose and text.strip():
            print(text)
    if failed:
        raise RuntimeError("nvcc failed for " + ", ".join(failed))
    tmp = LIB + ".tmp"
    subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    ex = ["-Xptxas", "-v"] if "--ptxas" in sys.argv else []
    print(build(force=True, verbose=v, extra=ex))
