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
