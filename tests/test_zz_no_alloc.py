"""sg_transport_bank_noalloc: the gen loop for callers that cannot allocate device memory.

Callers whose device memory belongs to another allocator or to a pool reserved up front, and
real-time sections that must not block in the driver's allocator, cannot call cudaMalloc while a
cycle runs.  This entry point keeps its scratch in
a static device array and works on banks the caller already holds on the device.  The test checks
that two calls in a row (the second one sees the first call's leftovers in the shared scratch) give
the fission bank of the allocating entry point, sg_transport_bank, within the parity tolerances.
The file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from scone_gb300 import abi, problems

pytestmark = pytest.mark.gpu

SEED = 0x5C3A84C9


def test_noalloc_gen_loop_matches_transport_bank_on_two_calls():
    import torch
    from scone_gb300 import gpu

    L = gpu.load()
    p = problems.lattice_17x17_7g()
    t = gpu.TransportOperatorGPU(p, precision=abi.PREC_FP64, form=abi.FORM_HISTORY, max_bank=1 << 16)
    adm = t.upload_tally(p.tallies["mesh"] + [abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
    n = 4000
    t.eigen_init(n, SEED)
    bank, pop = t.eigen_bank(n)
    assert pop == n
    cap = 16384
    ref, st = t.transport_bank(adm, bank, 777, k_eff=1.05, next_cap=cap)
    m = st.n_next
    assert m > 0

    # the caller's own device memory for the input and output banks
    dev = torch.device("cuda", 0)
    fin = {k: torch.from_numpy(np.ascontiguousarray(bank[k][:n])).to(dev) for k in ("wgt", "r", "dir", "G", "time")}
    fout = {k: torch.empty((cap, 3) if k in ("r", "dir") else (cap,),
                           dtype=torch.int32 if k in ("G", "brood_id") else torch.float64, device=dev)
            for k in ("wgt", "r", "dir", "G", "time", "brood_id")}
    dp = lambda x, ct: C.cast(C.c_void_p(x.data_ptr()), C.POINTER(ct))
    bin_ = abi.Bank(dp(fin["wgt"], C.c_double), dp(fin["r"], C.c_double), dp(fin["dir"], C.c_double),
                    dp(fin["G"], C.c_int32), dp(fin["time"], C.c_double), C.cast(None, C.POINTER(C.c_int32)))
    bout = abi.Bank(dp(fout["wgt"], C.c_double), dp(fout["r"], C.c_double), dp(fout["dir"], C.c_double),
                    dp(fout["G"], C.c_int32), dp(fout["time"], C.c_double), dp(fout["brood_id"], C.c_int32))
    torch.cuda.synchronize()
    for call in range(2):
        for v in fout.values():
            v.fill_(-1)
        torch.cuda.synchronize()
        n_next = C.c_int32(-1)
        rc = L.sg_transport_bank_noalloc(t.h, adm, C.byref(bin_), n, C.c_uint64(777), 1.05, C.byref(bout), cap,
                                         C.byref(n_next))
        assert rc == 0, t._check(rc)
        assert n_next.value == m, (call, n_next.value, m)
        got = {k: v[:m].cpu().numpy() for k, v in fout.items()}
        for k in ("G", "wgt", "brood_id"):
            assert np.array_equal(got[k], ref[k][:m]), (call, k)
        np.testing.assert_allclose(got["r"], ref["r"][:m], rtol=0, atol=1e-9)
        np.testing.assert_allclose(got["dir"], ref["dir"][:m], rtol=0, atol=1e-12)

    # sizes beyond the stated maximum are rejected, not run
    big = C.c_int32(0)
    rc = L.sg_transport_bank_noalloc(t.h, adm, C.byref(bin_), 16385, C.c_uint64(777), 1.05, C.byref(bout), cap,
                                     C.byref(big))
    assert rc == abi.SG_OK - 1   # SG_ERR_BAD_ARG
