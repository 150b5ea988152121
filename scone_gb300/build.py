"""Builds libsconegpu.so in-tree (scone_gb300/_build/) with nvcc for sm_103a.

Translation units compile in parallel: six per (nuclear data, precision form, transport operator)
for the transport kernels (sg_tr_unit.cu with the SG_* macros: history loop and event kernels, each
for nesting bounds 2, 3 and 4), one per (precision, operator) for the batched kernel, and the host and
support units.  The FP64 verification units and the support kernels are compiled with -fmad=false
(every multiply and add rounded separately, as SCONE's gfortran build does on x86-64); the
mixed-precision units keep FMA contraction.
"""
import os
import shutil
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsconegpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no multiply-add contraction (gcc contracts by default on aarch64), so host-side values
# such as rotation matrices are the same on every host and equal the oracle's
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
# (object name, source, flags)
UNITS = [(u.replace(".cu", ""), u, ["-fmad=false"])
         for u in ("sg_support.cu", "sg_host.cu", "sg_noalloc.cu", "sg_fission_source.cu", "sg_batch_host.cu")]
for _op in ("st", "dt", "ht"):
    for _prec, _R, _fl in (("fp64", "double", ["-fmad=false"]), ("mixed", "float", [])):
        for _data, _ce in (("mg", 0), ("ce", 1)):
            for _part in range(9 if _ce == 0 else 6):    # 6-8: the lean history loop, multigroup only
                UNITS.append((f"sg_tr_{_data}_{_prec}_{_op}_p{_part}", "sg_tr_unit.cu",
                              _fl + [f"-DSG_R={_R}", f"-DSG_CE={_ce}", f"-DSG_OP=OP_{_op.upper()}",
                                     f"-DSG_PART={_part}"]))
        UNITS.append((f"sg_batch_{_prec}_{_op}", f"sg_batch_{_prec}_{_op}.cu", _fl))


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


def _big_stack():
    """Compilers inherit the largest stack the hard limit allows: the front end recurses deeply on the
    biggest units, and an 8 MB stack has made it crash on aarch64 hosts."""
    try:
        import resource
        soft, hard = resource.getrlimit(resource.RLIMIT_STACK)
        resource.setrlimit(resource.RLIMIT_STACK, (hard, hard))
    except (ImportError, ValueError, OSError):
        pass


def build(force=False, verbose=False, extra=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    objs = []
    cmds = []
    for unit, src, flags in UNITS:
        obj = os.path.join(OUT, unit + ".o")
        cmds.append((unit, [cc, *ARCH, *COMMON, *flags, *extra, "-c", os.path.join(CSRC, src), "-o", obj]))
        objs.append(obj)
    # the long units first (history loops and event kernels of the hybrid operator, then the rest of
    # the transport parts, then the batched kernels), at most one compiler per host core
    cmds.sort(key=lambda c: (not c[0].endswith("_ht_p2") and not c[0].endswith("_ht_p3"),
                             not c[0].startswith("sg_tr_"), not c[0].startswith("sg_batch_")))
    jobs = max(1, os.cpu_count() or 1)
    failed = []
    running = []

    def finish(item):
        unit, p = item
        out, _ = p.communicate()
        running.remove(item)
        text = out.decode(errors="replace")
        if p.returncode != 0:
            failed.append(unit)
            sys.stderr.write(text)
        elif verbose and text.strip():
            print(text)

    def wait_one():
        while True:
            for item in running:
                if item[1].poll() is not None:
                    finish(item)
                    return
            time.sleep(0.1)

    for unit, cmd in cmds:
        if len(running) >= jobs:
            wait_one()
        if verbose:
            print(" ".join(cmd), flush=True)
        running.append((unit, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                               preexec_fn=_big_stack)))
    while running:
        wait_one()
    # a unit that failed while many compilers ran is compiled again on its own, up to three times (the
    # compiler has been seen to crash with SIGSEGV on aarch64 hosts, now and then, on units it
    # compiles cleanly otherwise); a real compile error fails every time and is reported
    retry = [(u, c) for u, c in cmds if u in failed]
    failed.clear()
    for unit, cmd in retry:
        for attempt in range(3):
            p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, preexec_fn=_big_stack)
            if p.returncode == 0:
                break
        if p.returncode != 0:
            failed.append(unit)
            sys.stderr.write(p.stdout.decode(errors="replace"))
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
