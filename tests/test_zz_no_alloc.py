"""sg_transport_bank_noalloc: the gen loop for callers that cannot allocate device memory.

Callers whose device memory belongs to another allocator or to a pool reserved up front, and
real-time sections that must not block in the driver's allocator, cannot call cudaMalloc while a
cycle runs.  This entry point keeps its scratch in a static device array and works on banks the
caller already holds on the device.  The tests check, through the C ABI, that two calls in a row
(the second one sees the first call's leftovers in the shared scratch) give the fission bank and
the tally bins of the allocating entry point, sg_transport_bank, in both precision forms; that a
call near the site limit succeeds and one beyond it fails cleanly (and the next call works again);
and that sizes beyond the stated maximum, and continuous-energy handles, are refused.
The file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from scone_gb300 import abi, problems

pytestmark = pytest.mark.gpu

SEED = 0x5C3A84C9
MAX_HIST = 16384
MAX_SITES = 32768
SG_ERR_BAD_ARG, SG_ERR_BANK_OVERFLOW, SG_ERR_STATE = -1, -3, -9


def _device_banks(torch, bank, n, cap):
    dev = torch.device("cuda", 0)
    fin = {k: torch.from_numpy(np.ascontiguousarray(bank[k][:n])).to(dev) for k in ("wgt", "r", "dir", "G", "time")}
    fout = {k: torch.empty((cap, 3) if k in ("r", "dir") else (cap,),
                           dtype=torch.int32 if k in ("G", "brood_id") else torch.float64, device=dev)
            for k in ("wgt", "r", "dir", "G", "time", "brood_id")}
    dp = lambda x, ct: C.cast(C.c_void_p(x.data_ptr()), C.POINTER(ct))
    none = C.cast(None, C.POINTER(C.c_int32))
    bin_ = abi.Bank(dp(fin["wgt"], C.c_double), dp(fin["r"], C.c_double), dp(fin["dir"], C.c_double),
                    dp(fin["G"], C.c_int32), dp(fin["time"], C.c_double), none)
    bout = abi.Bank(dp(fout["wgt"], C.c_double), dp(fout["r"], C.c_double), dp(fout["dir"], C.c_double),
                    dp(fout["G"], C.c_int32), dp(fout["time"], C.c_double), dp(fout["brood_id"], C.c_int32))
    return fin, fout, bin_, bout


def _noalloc(L, t, adm, bin_, n, master, k, bout, cap):
    n_next = C.c_int32(-1)
    rc = L.sg_transport_bank_noalloc(t.h, adm, C.byref(bin_), n, C.c_uint64(master), k, C.byref(bout), cap,
                                     C.byref(n_next))
    return rc, n_next.value


def _check_bank(got, ref, m, exact_r):
    for k in ("G", "wgt", "brood_id"):
        assert np.array_equal(got[k][:m], ref[k][:m]), k
    if exact_r:
        assert np.array_equal(got["r"][:m], ref["r"][:m])
        assert np.array_equal(got["dir"][:m], ref["dir"][:m])
    else:
        np.testing.assert_allclose(got["r"][:m], ref["r"][:m], rtol=0, atol=1e-9)
        np.testing.assert_allclose(got["dir"][:m], ref["dir"][:m], rtol=0, atol=1e-12)


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_noalloc_gen_loop_matches_transport_bank_on_two_calls(precision):
    import torch
    from scone_gb300 import gpu

    L = gpu.load()
    p = problems.lattice_17x17_7g()
    t = gpu.TransportOperatorGPU(p, precision=precision, form=abi.FORM_HISTORY, max_bank=1 << 16)
    clerks = p.tallies["mesh"] + [abi.clerk(abi.CLERK_KEFF_IMPLICIT)]
    adm_ref = t.upload_tally(clerks)
    adm_na = t.upload_tally(clerks)
    n = 4000
    t.eigen_init(n, SEED)
    bank, pop = t.eigen_bank(n)
    assert pop == n
    cap = 16384
    fin, fout, bin_, bout = _device_banks(torch, bank, n, cap)
    torch.cuda.synchronize()
    for call, master in enumerate((777, 778)):
        # the allocating entry point: the reference for this call
        ref, st = t.transport_bank(adm_ref, bank, master, k_eff=1.05, next_cap=cap)
        t.tally_cycle_end(adm_ref, float(st.n_next), 1.05)
        m = st.n_next
        assert m > 0
        for v in fout.values():
            v.fill_(-1)
        torch.cuda.synchronize()
        rc, n_next = _noalloc(L, t, adm_na, bin_, n, master, 1.05, bout, cap)
        assert rc == 0, t._check(rc)
        assert n_next == m, (call, n_next, m)
        got = {k: v[:m].cpu().numpy() for k, v in fout.items()}
        _check_bank(got, ref, m, exact_r=True)
        t.tally_cycle_end(adm_na, float(m), 1.05)
        # the same scores; the FP64 sums differ only in the order of their atomic additions
        np.testing.assert_allclose(t.bins(adm_na), t.bins(adm_ref), rtol=1e-10, atol=1e-300)
    # sizes beyond the stated maximum are rejected, not run
    rc, _ = _noalloc(L, t, adm_na, bin_, MAX_HIST + 1, 777, 1.05, bout, cap)
    assert rc == SG_ERR_BAD_ARG
    t.close()


def test_noalloc_site_limit_is_the_call_total():
    """A call whose fission sites come close to SG_NOALLOC_MAX_SITES succeeds and equals the
    allocating entry point; one that makes more fails with SG_ERR_BANK_OVERFLOW without writing out
    of bounds, and the next call works again."""
    import torch
    from scone_gb300 import gpu

    L = gpu.load()
    p = problems.lattice_17x17_7g()
    t = gpu.TransportOperatorGPU(p, precision=abi.PREC_FP64, form=abi.FORM_HISTORY, max_bank=1 << 17)
    clerks = p.tallies["mesh"] + [abi.clerk(abi.CLERK_KEFF_IMPLICIT)]
    adm_ref, adm_na, adm_bad = (t.upload_tally(clerks) for _ in range(3))
    n = MAX_HIST
    t.eigen_init(n, SEED)
    bank, pop = t.eigen_bank(n)
    assert pop == n
    cap = 1 << 17
    # k_eff scales the sites per history (n = int(w nuSigma_f / (w0 Sigma_t k) + xi)); the allocating
    # path gives each k's site count
    sites = {}
    for k in np.linspace(0.40, 0.80, 41):
        _, st = t.transport_bank(adm_ref, bank, 4242, k_eff=float(k), next_cap=cap)
        sites[float(k)] = st.n_next
    near = [k for k, s in sites.items() if 0.9 * MAX_SITES <= s <= MAX_SITES]
    over = [k for k, s in sites.items() if s > MAX_SITES]
    assert near and over, sites
    k_near, k_over = max(near, key=lambda k: sites[k]), max(over)
    fin, fout, bin_, bout = _device_banks(torch, bank, n, cap)
    torch.cuda.synchronize()
    ref, st = t.transport_bank(adm_ref, bank, 4242, k_eff=k_near, next_cap=cap)
    rc, n_next = _noalloc(L, t, adm_na, bin_, n, 4242, k_near, bout, cap)
    assert rc == 0, t._check(rc)
    assert n_next == st.n_next == sites[k_near]
    _check_bank({k: v[:n_next].cpu().numpy() for k, v in fout.items()}, ref, n_next, exact_r=True)
    rc, _ = _noalloc(L, t, adm_bad, bin_, n, 4242, k_over, bout, cap)
    assert rc == SG_ERR_BANK_OVERFLOW
    buf = C.create_string_buffer(256)
    L.sg_last_error(t.h, buf, 256)
    assert b"SG_NOALLOC_MAX_SITES" in buf.value
    rc, n_next = _noalloc(L, t, adm_na, bin_, n, 4242, k_near, bout, cap)
    assert rc == 0 and n_next == sites[k_near]
    _check_bank({k: v[:n_next].cpu().numpy() for k, v in fout.items()}, ref, n_next, exact_r=True)
    t.close()


def test_noalloc_refuses_continuous_energy_handles():
    import torch
    from scone_gb300 import gpu

    L = gpu.load()
    p = problems.ce_slab_3layer(points=(2000, 4000))
    t = gpu.TransportOperatorGPU(p, precision=abi.PREC_FP64, form=abi.FORM_HISTORY, max_bank=1 << 12)
    adm = t.upload_tally(p.tallies["flux"])
    bank = t.generate_source(SEED, 64)
    fin, fout, bin_, bout = _device_banks(torch, bank, 64, 256)
    rc, _ = _noalloc(L, t, adm, bin_, 64, 1, 1.0, bout, 256)
    assert rc == SG_ERR_STATE
    buf = C.create_string_buffer(256)
    L.sg_last_error(t.h, buf, 256)
    assert b"multigroup" in buf.value
    t.close()
