"""The C-ABI library builds, loads without a GPU and exports every entry point of include/scone_gpu.h."""
import ctypes
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "scone_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int32_t|uint64_t|double)\s+(sg_\w+)\s*\(", text, re.M)))


def test_library_exports_all_declared_symbols():
    from scone_gb300 import gpu
    L = gpu.load()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s


def test_host_rng_entry_points_match_oracle(oracle_mod):
    from scone_gb300 import gpu
    a, sa = gpu.rng_draws(0x5C3A84C9, 100)
    b, sb = oracle_mod.rng_draws(0x5C3A84C9, 100)
    assert np.array_equal(a, b) and sa == sb
    for k in (1, 152917, 13456757, -13456758, 2**40 + 3):
        assert gpu.rng_skip(12345, k) == oracle_mod.rng_skip(12345, k)


def test_create_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        return
    from scone_gb300 import gpu, abi
    try:
        gpu.TransportOperatorGPU(max_bank=16, precision=abi.PREC_FP64)
    except gpu.SconeGpuError:
        return
    raise AssertionError("creating a handle without a GPU must raise")


def test_bank_file_round_trip(tmp_path):
    """particleDungeon%printToFile layout (10 doubles per particle: r, dir, E, G, broodID, wgt) written
    and read back by the library's host code, in binary and text form; no GPU is involved."""
    from scone_gb300 import abi, gpu
    rng = np.random.default_rng(9)
    n = 257
    b = abi.HostBank(n)
    b["r"][:] = rng.normal(size=(n, 3))
    d = rng.normal(size=(n, 3))
    b["dir"][:] = d / np.linalg.norm(d, axis=1)[:, None]
    b["wgt"][:] = rng.uniform(0.5, 2.0, n)
    b["G"][:] = rng.integers(1, 8, n)
    b["brood_id"][:] = np.arange(1, n + 1)
    b["E"][:] = rng.uniform(1e-9, 10.0, n)
    for binary in (True, False):
        stem = str(tmp_path / ("bank" + str(binary)))
        gpu.write_bank_file(stem, b, binary=binary)
        path = stem + (".bin" if binary else ".txt")
        if binary:
            raw = np.fromfile(path, dtype=np.float64).reshape(n, 10)
            np.testing.assert_array_equal(raw[:, 0:3], b["r"])
            np.testing.assert_array_equal(raw[:, 7], b["G"].astype(float))
            np.testing.assert_array_equal(raw[:, 9], b["wgt"])
        c = gpu.read_bank_file(path, binary=binary)
        assert c.n == n
        for k in ("r", "dir", "wgt", "E"):
            np.testing.assert_array_equal(c[k], b[k])
        np.testing.assert_array_equal(c["G"], b["G"])
        np.testing.assert_array_equal(c["brood_id"], b["brood_id"])


STRUCTS = {"GeometryDesc": "sg_geometry_desc", "MGDesc": "sg_mg_desc", "CEDesc": "sg_ce_desc",
           "AxisDesc": "sg_axis_desc", "ClerkDesc": "sg_clerk_desc", "TallyDesc": "sg_tally_desc",
           "PointSourceDesc": "sg_point_source_desc", "Config": "sg_config", "Bank": "sg_bank",
           "CycleStats": "sg_cycle_stats", "CollisionDesc": "sg_collision_desc", "EventTuning": "sg_event_tuning",
           "BatchConfig": "sg_batch_config", "ProblemDesc": "sg_problem_desc", "BatchTuning": "sg_batch_tuning",
           "BatchStats": "sg_batch_stats"}


def test_python_structs_match_the_header(tmp_path):
    """Every ctypes mirror in scone_gb300/abi.py has the size and field offsets of its struct in
    include/scone_gpu.h (a C program built with the host compiler prints them)."""
    import shutil
    import subprocess
    from scone_gb300 import abi
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "scone_gpu.h"', 'int main(void) {']
    for py, c in STRUCTS.items():
        lines.append(f'  printf("{py} size %zu\\n", sizeof({c}));')
        for name, _ in getattr(abi, py)._fields_:
            lines.append(f'  printf("{py} {name} %zu\\n", offsetof({c}, {name}));')
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for py in STRUCTS:
        cls = getattr(abi, py)
        assert got[(py, "size")] == ctypes.sizeof(cls), py
        for name, _ in cls._fields_:
            assert got[(py, name)] == getattr(cls, name).offset, (py, name)
