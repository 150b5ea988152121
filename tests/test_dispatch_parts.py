"""The launch of a transport kernel reaches the part (translation unit) that holds it: the history
loop or the event kernels, for nesting bound 2, 3 or 4, and a multigroup history loop whose launch
is lean the lean instantiation (parts 6-8; scone_gb300/csrc/sg_launch.h).  A host program built with
the host compiler replaces the parts with recorders; no GPU is used."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROG = r'''
#include <cstdio>
#include "sg_launch.h"
namespace sg {
static int last = -1;
#define PART(R, CE, OP, P) template <> cudaError_t launch_part<R, CE, OP, P>(int, const TransportArgs<R>&, size_t, \
    cudaStream_t, int*) { last = 1000 * (sizeof(R) == 8) + 100 * CE + 10 * OP + P; return cudaSuccess; }
#define PARTS(R, CE, OP) PART(R, CE, OP, 0) PART(R, CE, OP, 1) PART(R, CE, OP, 2) PART(R, CE, OP, 3) \
    PART(R, CE, OP, 4) PART(R, CE, OP, 5)
#define LEAN(R, OP) PART(R, false, OP, 6) PART(R, false, OP, 7) PART(R, false, OP, 8)
#define OPS(R, CE) PARTS(R, CE, OP_ST) PARTS(R, CE, OP_DT) PARTS(R, CE, OP_HT)
OPS(float, false) OPS(float, true) OPS(double, false) OPS(double, true)
LEAN(float, OP_ST) LEAN(float, OP_DT) LEAN(float, OP_HT) LEAN(double, OP_ST) LEAN(double, OP_DT) LEAN(double, OP_HT)
}
int main() {
  sg::TransportArgs<float> a{};
  sg::TransportArgs<double> b{};
  const int kinds[5] = {sg::K_HISTORY, sg::K_EV_START, sg::K_EV_TRANSIT, sg::K_EV_COLLIDE, sg::K_EV_TAIL};
  for (int maxl : {2, 3, 4})
    for (int op : {sg::OP_ST, sg::OP_DT, sg::OP_HT})
      for (int kind : kinds)
        for (int lean : {0, 1}) {
          a.lean = b.lean = lean;
          sg::launch_kind_data<float, false>(kind, a, maxl, op, 0, nullptr, nullptr);
          std::printf("f 0 %d %d %d %d %d\n", maxl, op, kind, lean, sg::last);
          sg::launch_kind_data<double, true>(kind, b, maxl, op, 0, nullptr, nullptr);
          std::printf("d 1 %d %d %d %d %d\n", maxl, op, kind, lean, sg::last);
        }
  return 0;
}
'''


def test_launch_reaches_its_part(tmp_path):
    cxx = shutil.which("g++")
    inc = "/usr/local/cuda/include"
    if cxx is None or not os.path.exists(os.path.join(inc, "cuda_runtime.h")):
        pytest.skip("no host compiler or CUDA headers")
    src = tmp_path / "parts.cpp"
    src.write_text(PROG)
    exe = tmp_path / "parts"
    subprocess.run([cxx, "-std=c++17", "-I", inc, "-I", os.path.join(ROOT, "scone_gb300", "csrc"), str(src), "-o",
                    str(exe)], check=True)
    rows = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    seen = 0
    for r in rows:
        if not r.strip():
            continue
        prec, ce, maxl, op, kind, lean, got = r.split()
        maxl, op, kind, lean, got = int(maxl), int(op), int(kind), int(lean), int(got)
        part = (0 if maxl <= 2 else (2 if maxl == 3 else 4)) + (0 if kind == 0 else 1)
        if lean and kind == 0 and ce == "0":              # the lean history loop: multigroup only
            part = 6 + (0 if maxl <= 2 else (1 if maxl == 3 else 2))
        want = 1000 * (prec == "d") + 100 * int(ce) + 10 * op + part
        assert got == want, r
        seen += 1
    assert seen == 3 * 3 * 5 * 2 * 2
