#!/usr/bin/env python3
"""Benchmark of the SCONE particle-tracking cycle on GB300.

Workload: the 17x17 pin-lattice k-eigenvalue problem (7 groups, seeded synthetic XS, pitch 1.26 cm,
pin radius 0.54 cm, reflective box), 1e6 particles per cycle, delta tracking (surface tracking
measured beside it), FP32 XS/distances with FP64 positions and tally sums.  One step = one active
eigenvalue cycle on a converged bank: the gen loop over the bank, fission-site ordering, tally cycle
end (17x17x7 mesh flux + implicit k), normSize_Repr and k feedback.

  value  histories/s of the device-resident cycle (CUDA events on the library's stream)
  e2e    histories/s of the same cycle through the C ABI with host banks (sg_eigen_cycle_bank): the
         bank in page-locked host memory, read by the kernels across the host link, and the
         normalised next bank copied back to the host, inside every step
  roofline  the history-loop kernel: algorithmic bytes (128 B per event, mixed form) / kernel time,
         with the compute-side counters of its committed ncu capture
  cpu_baseline  the same eigenvalue cycle of SCONE's algorithm on the host cores (the oracle's OpenMP
         cycle, the code `--impl reference` times), bounded sample

Beside the lattice line, the same JSON line carries config 1's k and mesh-flux deviation of the
mixed form from the all-FP64 form (50 inactive + 100 active cycles of 1e6), the infinite medium and
the CE slab (each with its tally deviation from FP64), and the uneven batch (4096 independent
fixed-source problems of 1-16 groups, spheres and multi-slabs, 1e3-1e6 histories each, 5.9e8
histories in all):

  batched   histories/s of the batched form (every cycle of every problem in one persistent launch,
            one CUDA graph), mixed precision, delta tracking, launch shape from the autotuner
  plain     histories/s of the plain form over the same batch: one problem per launch sequence
            (sg_fixed_source_cycle per cycle), event-based and history-loop kernels; compared
            device time with device time and wall clock with wall clock
  tally error  per-bin relative errors of the batched mixed form against the all-FP64 batched form
  cpu_baseline  a stratified, timed sample of the 4096 problems run one after another through the
            oracle (OpenMP over histories), extrapolated to the whole batch
  serving   Poisson arrivals of requests drawn from the batch (plus 5 % lattice eigenvalue
            requests), continuous batching: p50/p99 latency, achieved and offered histories/s,
            per-request tally error against the all-FP64 form

`--impl reference` times SCONE's algorithm on the host cores instead (the oracle restatement: SCONE
itself is Fortran and cannot be built here), on the same workload, step and metric.
Multi-GPU (torchrun): independent replicas, one per rank, each with its own RNG offset (the path
shards over histories with no exchange inside a cycle); value sums all ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_EVENT_MIXED = 128   # r 24 + u 12 + w 4 + rng 8 + (G, mat, cell/lattice) 8 = 56 B, x2, + 16 B tally RMW
BYTES_PER_EVENT_FP64 = 176
SEED = 0x5C3A84C9


def args_():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--pop", type=int, default=None, help="particles per cycle (default 1e6; 1e5 with --profile)")
    ap.add_argument("--transport", default="dt", choices=["st", "dt", "st-nocache"])
    ap.add_argument("--no-alt", action="store_true", help="skip the second transport operator measurement")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--form", default="history", choices=["event", "history"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--profile", action="store_true", help="a short run for ncu captures")
    ap.add_argument("--batch-problems", type=int, default=4096, help="problems of the uneven batch")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched / plain / served measurements")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain one-problem-per-launch forms")
    ap.add_argument("--no-fp64-batch", action="store_true", help="skip the all-FP64 batched reference run")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--wave-histories", type=int, default=1 << 23, help="histories per serving wave")
    ap.add_argument("--serve-item", type=int, default=256, help="histories per work item while serving")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shape of the batch")
    ap.add_argument("--no-configs", action="store_true", help="skip the infinite-medium and CE-slab lines")
    a = ap.parse_args()
    if a.profile:   # a reduced run for ncu captures: lattice cycles, one small batch and one CE cycle
        a.no_cpu_baseline = a.no_e2e = a.no_alt = a.no_plain = a.no_fp64_batch = a.no_serve = True
        a.no_autotune = a.no_configs = True
        a.batch_problems = min(a.batch_problems, 256)
    if a.pop is None:
        a.pop = 100_000 if a.profile else 1_000_000
    return a


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(kernel):
    """Measured DRAM bytes per event of `kernel` (an ncu capture summarised under profiles/)."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f).get(kernel, {}).get("bytes_per_event")
    return None


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def lattice_setup(t, p):
    from scone_gb300 import abi
    inact = t.upload_tally([])
    act = t.upload_tally(p.tallies["mesh"])
    ia = t.upload_tally([abi.clerk(abi.CLERK_KEFF_ANALOG)])
    aa = t.upload_tally([abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
    t.attach_tally(inact, ia)
    t.attach_tally(act, aa)
    return inact, ia, act, aa


def transport_code(a):
    from scone_gb300 import abi
    return {"st": abi.TRANSPORT_ST, "dt": abi.TRANSPORT_DT, "st-nocache": abi.TRANSPORT_ST_NOCACHE}[a.transport]


def workload_config(a, world):
    """The workload and step both arms time, as one dict (the reference arm prints the same one)."""
    return {"workload": "lattice_17x17_7g_eigen", "particles_per_cycle": a.pop, "groups": 7,
            "lattice": "17x17 pins r=0.54 cm pitch=1.26 cm, reflective box", "transport": a.transport.upper(),
            "step": "one active eigenvalue cycle on a converged bank: gen loop, fission-site order, tally cycle "
                    "end, normSize_Repr, k feedback",
            "warmup_cycles": "inactive cycles (keff analog tally) before the timed active cycles",
            "tally": "17x17x7 mesh flux (collision estimator) + implicit k",
            "l2": "per-step working set exceeds L2 (bank 72 MB in, ~80 MB sites, 72 MB ordered, 72 MB normalised)",
            "parallelism": f"replicas{world}"}


def cpu_eigen_cycles(p, pop, transport, threads, inactive, active=None, target_s=None):
    """SCONE's eigenvalue cycle on the host cores: the oracle's OpenMP cycle (histories over threads,
    thread-private score memory summed at the cycle end, sites ordered by brood, cycle end,
    normSize_Repr and k feedback on the master thread) after `inactive` cycles from the fission
    source; then `active` timed cycles, or as many as fit in target_s seconds.
    Returns (seconds per timed cycle, events per timed cycle, histories per cycle)."""
    from oracle import oracle
    o = oracle.Oracle(p, transport=transport)
    inact, ia, act, aa = lattice_setup(o, p)
    o.eigen_init(pop, SEED)
    for _ in range(inactive):
        o.eigen_cycle_omp(inact, ia, threads)
    secs, evs = [], []
    t_start = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        st = o.eigen_cycle_omp(act, aa, threads)
        secs.append(time.perf_counter() - t0)
        evs.append(st.n_events)
        if active is not None and len(secs) >= active:
            break
        if target_s is not None and time.perf_counter() - t_start >= target_s:
            break
    o.close()
    return secs, evs, pop


def host_bank_dict(b, n):
    return {k: b[k][:n].copy() for k in ("wgt", "r", "dir", "G", "time", "brood_id")}


def link_d2h_gbps(nbytes, reps=5):
    """The host link's device-to-host copy rate for one pinned copy of nbytes (CUDA events around a
    torch copy): what the end-to-end call's copy back of the normalised bank can reach."""
    import torch
    dev = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    host = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    best = None
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        host.copy_(dev, non_blocking=True)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    del dev, host
    return nbytes / best / 1e6


def pinned_bank(src, n, cap):
    """A HostBank in page-locked host memory (cudaHostAlloc through torch), filled from src."""
    import torch
    from scone_gb300 import abi
    arrs = {}
    for k, shape, dt in (("wgt", (cap,), torch.float64), ("r", (cap, 3), torch.float64),
                         ("dir", (cap, 3), torch.float64), ("G", (cap,), torch.int32),
                         ("time", (cap,), torch.float64), ("brood_id", (cap,), torch.int32)):
        t = torch.zeros(shape, dtype=dt).pin_memory()
        if src is not None:
            t[:n].copy_(torch.from_numpy(src[k][:n].copy()))
        arrs[k] = t
    hb = abi.HostBank(cap, {k: v.numpy() for k, v in arrs.items()})
    hb.pinned = arrs
    return hb


def reference_arm(a, p):
    """SCONE's algorithm on the host cores (the oracle's OpenMP eigenvalue cycle), same workload,
    step and metric as the GPU arm: the same number of inactive cycles, then K timed active cycles."""
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    warm = max(3, a.warmup)
    secs, evs, n = cpu_eigen_cycles(p, a.pop, transport_code(a), threads, warm, active=a.steps)
    tot = sum(secs)
    value = a.steps * n / tot
    line = {
        "impl": "reference", "metric": "histories/s", "value": value, "unit": "histories/s",
        "n_gpus": a.gpus, "steps": a.steps, "warmup": warm, "ms_per_step": 1e3 * tot / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "events_per_s": sum(evs) / tot,
        "config": workload_config(a, world),
        "reference": "C++ restatement of SCONE's algorithm (oracle/), OpenMP over histories as SCONE's OpenMP "
                     "build; SCONE is Fortran and no Fortran compiler exists here",
        "cpu_baseline": {"value": value, "unit": "histories/s", "cores": threads, "kind": "port",
                         "sample": f"{warm} inactive + {a.steps} timed active cycles of {n} particles, "
                                   f"OpenMP over histories on {threads} threads"},
        "e2e": {"value": value, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


def tally_deviation(b64, b32, n_batches):
    """Per-bin deviation of a mixed-form tally from the all-FP64 one (scoreMemory bins(N,3) of both,
    n_batches batches): z = mean difference / combined sigma, and the ratio of the relative
    standard errors (mixed / FP64)."""
    import numpy as np
    n = n_batches
    m1, m2 = b64[:, 1] / n, b32[:, 1] / n
    v1 = np.maximum(b64[:, 2] / n - m1 ** 2, 0) / (n - 1)
    v2 = np.maximum(b32[:, 2] / n - m2 ** 2, 0) / (n - 1)
    ok = (v1 > 0) & (v2 > 0) & (m1 > 0) & (m2 > 0)
    if not ok.any():
        return {"bins": 0}
    z = (m2[ok] - m1[ok]) / np.sqrt(v1[ok] + v2[ok])
    ratio = (np.sqrt(v2[ok]) / m2[ok]) / (np.sqrt(v1[ok]) / m1[ok])
    dev = np.abs(ratio - 1.0)
    return {"bins": int(ok.sum()), "z_mean": float(z.mean()), "z_std": float(z.std()),
            "max_abs_z": float(np.abs(z).max()), "chi2_per_bin": float(np.mean(z ** 2)),
            "rel_err_ratio_median_abs_dev": float(np.median(dev)), "rel_err_ratio_p99_abs_dev": float(np.percentile(dev, 99)),
            "frac_rel_err_within_10pct": float(np.mean(dev < 0.10)),
            "note": "both forms draw the same RNG streams, so most histories follow the same path and the "
                    "differences are far smaller than independent runs would show"}


def lattice_k_section(a, local, inactive=50, active=100, pop=1_000_000, replicas=6):
    """Config 1 as stated: k and the 17x17x7 mesh flux of the mixed form against the all-FP64 form,
    each from `replicas` independent runs (different seeds) of `inactive` + `active` cycles of 1e6
    particles (delta tracking).  The spread of the replicas' results is the uncertainty: the
    cycle-to-cycle sigma of one run underestimates it, because the fission source of an eigenvalue
    run is correlated from cycle to cycle (the ratio of the two is reported)."""
    import numpy as np
    from scone_gb300 import abi, gpu, problems
    p = problems.lattice_17x17_7g()
    res = {}
    for name, prec in (("mixed", abi.PREC_MIXED), ("fp64", abi.PREC_FP64)):
        t = gpu.TransportOperatorGPU(p, precision=prec, transport=abi.TRANSPORT_DT, max_bank=int(2.5 * pop) + 4096,
                                     device=local, form=abi.FORM_HISTORY)
        ks, sds, mesh = [], [], []
        t0 = time.perf_counter()
        for r in range(replicas):
            inact, ia, act, aa = lattice_setup(t, p)
            t.eigen_init(pop, gpu.rng_skip(SEED, 7919 * 152917 * (r + 1) * pop))
            for _ in range(inactive):
                t.eigen_cycle(inact, ia)
            for _ in range(active):
                t.eigen_cycle(act, aa)
            k, sd = t.keff(aa)
            ks.append(k)
            sds.append(sd)
            mesh.append(t.bins(act))
        res[name] = (np.array(ks), np.array(sds), np.array(mesh), time.perf_counter() - t0)
        t.close()
    (km, sm, mm, wm), (kd, sd, md, wd) = res["mixed"], res["fp64"]
    se_m, se_d = km.std(ddof=1) / np.sqrt(replicas), kd.std(ddof=1) / np.sqrt(replicas)
    z = (km.mean() - kd.mean()) / np.sqrt(se_m ** 2 + se_d ** 2)
    # relative standard error of each bin within one run (100 active cycles), averaged over the
    # replicas: the quantity the 10 % criterion compares
    def rel_err(b):
        m = b[:, :, 1] / active
        v = np.maximum(b[:, :, 2] / active - m ** 2, 0) / (active - 1)
        with np.errstate(divide="ignore", invalid="ignore"):
            return np.where(m > 0, np.sqrt(v) / m, np.nan).mean(axis=0)
    re_m, re_d = rel_err(mm), rel_err(md)
    # mesh flux: per bin, replica means and their standard errors
    mm, md = mm[:, :, 1] / active, md[:, :, 1] / active
    mmean, dmean = mm.mean(axis=0), md.mean(axis=0)
    mse, dse = mm.std(axis=0, ddof=1) / np.sqrt(replicas), md.std(axis=0, ddof=1) / np.sqrt(replicas)
    ok = (mse > 0) & (dse > 0) & (dmean > 0)
    zb = (mmean[ok] - dmean[ok]) / np.sqrt(mse[ok] ** 2 + dse[ok] ** 2)
    ratio = re_m[ok] / re_d[ok]
    return {"k_mixed": float(km.mean()), "se_mixed": float(se_m), "k_fp64": float(kd.mean()), "se_fp64": float(se_d),
            "z": float(z), "within_3_sigma": bool(abs(z) < 3.0),
            "replicas": replicas, "k_replicas": {"mixed": km.tolist(), "fp64": kd.tolist()},
            "sigma_ratio_replicas_over_within_run": float(np.sqrt((km.var(ddof=1) + kd.var(ddof=1)) / 2) /
                                                          np.mean(np.concatenate([sm, sd]))),
            "cycles": f"{replicas} independent runs per form of {inactive} inactive + {active} active cycles, "
                      f"{pop} particles, DT", "wall_s": {"mixed": wm, "fp64": wd},
            "mesh_flux_vs_fp64": {"bins": int(ok.sum()), "z_mean": float(zb.mean()), "z_std": float(zb.std()),
                                  "max_abs_z": float(np.abs(zb).max()), "chi2_per_bin": float(np.mean(zb ** 2)),
                                  "rel_err_ratio_median_abs_dev": float(np.median(np.abs(ratio - 1))),
                                  "frac_rel_err_within_10pct": float(np.mean(np.abs(ratio - 1) < 0.10)),
                                  "note": "z from the replica spread per bin; the relative-error ratio (mixed / "
                                          "FP64) from each run's cycle-to-cycle estimate, averaged over the "
                                          "replicas"}}


def configs_section(a, local):
    """The other two workloads, each through sg_fixed_source_cycle on its own handle (device-resident
    source, gen loop and batch close) and through the oracle on the host cores:
    infinite homogeneous medium, 2 groups, 1e5 histories; continuous-energy 3-layer slab, 1e7
    histories (10 cycles of 1e6), FP32 tables with FP64 energy and position.  Each carries the
    deviation of its tally in the mixed form from the all-FP64 form (same cycles, same seeds)."""
    from oracle import oracle
    from scone_gb300 import abi, gpu, problems
    threads = os.cpu_count() or 1
    out = {}
    cases = [("infinite_medium_2g", problems.infinite_medium_2g(), "flux", 100000, 1, 10, abi.TRANSPORT_ST),
             ("ce_slab_3layer", problems.ce_slab_3layer(), "current", 1000000, 10, 10, abi.TRANSPORT_DT)]
    for name, p, tally, pop, cycles, dev_cycles, tr in cases:
        res = {"histories": pop * cycles, "transport": "ST" if tr == abi.TRANSPORT_ST else "DT"}
        bins = {}
        for prec_name, prec in (("mixed", abi.PREC_MIXED), ("fp64", abi.PREC_FP64)):
            t = gpu.TransportOperatorGPU(p, precision=prec, transport=tr, max_bank=pop + 4096, device=local,
                                         form=abi.FORM_HISTORY)
            warm_adm = t.upload_tally(p.tallies[tally])
            adm = t.upload_tally(p.tallies[tally])
            t.fixed_source_cycle(warm_adm, min(pop, 10000), SEED)          # warm-up (own tally)
            m = SEED
            ms = ev = kms = 0.0
            for _ in range(cycles):
                m, st = t.fixed_source_cycle(adm, pop, m)
                ms += st.cycle_ms
                kms += st.transport_ms
                ev += st.n_events
            res[prec_name] = {"value": pop * cycles / (ms / 1e3), "unit": "histories/s",
                              "events_per_s": ev / (ms / 1e3), "ms": ms, "transport_kernel_ms": kms}
            if name.startswith("ce") and prec == abi.PREC_MIXED:
                # CE bytes per event: state 176 B + FP64 energy 16 B + per nuclide (hash bin, two grid
                # energies, two totals) 28 B x 10 + the sampled nuclide's pair 16 B
                peak, kind = measured_peaks()
                bpe = 176 + 16 + 28 * 10 + 16
                ach = ev * bpe / (kms / 1e3) / 1e9
                bpe_dram = committed_traffic("k_transport_ce_slab")
                res["roofline"] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                                   "peak_source": kind, "kernel": "k_transport<float, 2, DT, CE> (history loop)",
                                   "bytes_per_event": bpe, "events_per_launch": ev / cycles,
                                   "launch_ms": kms / cycles,
                                   "traffic": bpe_dram * ev / cycles if bpe_dram else None}
                comp = committed_compute("k_transport_ce_slab")
                if comp:
                    res["roofline"]["compute"] = comp
            # tally deviation: dev_cycles batches (more than the timed cycles when those are fewer)
            if dev_cycles > cycles:
                adm = t.upload_tally(p.tallies[tally])
                m = SEED
                for _ in range(dev_cycles):
                    m, _ = t.fixed_source_cycle(adm, pop, m)
            bins[prec_name] = t.bins(adm)
            t.close()
        res["tally_vs_fp64"] = tally_deviation(bins["fp64"], bins["mixed"], max(cycles, dev_cycles))
        res["tally_vs_fp64"]["tally"] = tally
        # the oracle on the host cores, a bounded sample (about 10 s)
        o = oracle.Oracle(p, transport=tr)
        adm = o.upload_tally(p.tallies[tally])
        n = min(pop, 200000 if name.startswith("ce") else 1000000)
        bank = o.generate_source(SEED, n)
        hist = ev = 0
        t0 = time.perf_counter()
        rep = 0
        while time.perf_counter() - t0 < 10.0:
            nh, e = o.timed_gen_loop(adm, bank, 4242 + rep, 1.0, threads)
            hist += nh
            ev += e
            rep += 1
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": hist / dt, "unit": "histories/s", "cores": threads, "kind": "port",
                               "sample": f"{hist} histories ({rep} x the gen loop over {n} source particles), "
                                         f"{dt:.1f} s"}
        res["speedup_mixed_vs_cpu"] = res["mixed"]["value"] / res["cpu_baseline"]["value"]
        out[name] = res
    return out


def batch_cpu_baseline(batch, threads, target_s=20.0, strata=8, seed=5):
    """The uneven batch on the host cores, as separate runs one after another (the plain CPU analogue
    of the batch): a stratified, timed sample.  Problems are sorted by history count into `strata`
    strata of equal size; from each, problems drawn at random (seeded) run through the oracle -- set
    up (geometry, data, tally), then every cycle: the point source and the gen loop with OpenMP over
    histories -- until the stratum has used its share of target_s.  The whole batch's time is
    estimated as the sum over strata of (mean seconds per sampled problem) x (problems in it)."""
    import numpy as np
    from oracle import oracle
    from scone_gb300 import abi
    hist = np.array([pop * c for _, pop, c, _ in batch], dtype=np.float64)
    groups = np.array_split(np.argsort(hist, kind="stable"), strata)
    rng = np.random.default_rng(seed)
    est = 0.0
    n_sampled = 0
    h_sampled = 0.0
    t_sampled = 0.0
    per_stratum = []
    for g in groups:
        times = []
        t_s = time.perf_counter()
        for i in rng.permutation(g):
            p, pop, cycles, master = batch[int(i)]
            t0 = time.perf_counter()
            o = oracle.Oracle(p, transport=abi.TRANSPORT_DT)
            adm = o.upload_tally(p.tallies["flux"])
            m = master
            for c in range(cycles):
                bank = o.generate_source(m, pop)
                o.timed_gen_loop(adm, bank, m + 1, 1.0, threads)
                m = oracle.rng_skip(m, 2 * 152917 * pop)
            o.close()
            times.append(time.perf_counter() - t0)
            h_sampled += hist[int(i)]
            if time.perf_counter() - t_s >= target_s / strata:
                break
        est += float(np.mean(times)) * len(g)
        n_sampled += len(times)
        t_sampled += float(np.sum(times))
        per_stratum.append({"problems": len(g), "sampled": len(times), "histories_min": float(hist[g].min()),
                            "histories_max": float(hist[g].max()), "mean_s_per_problem": float(np.mean(times))})
    return {"value": float(hist.sum()) / est, "unit": "histories/s", "cores": threads, "kind": "port",
            "estimated_batch_s": est,
            "sample": f"{n_sampled} of {len(batch)} problems ({h_sampled:.3g} histories, {t_sampled:.1f} s), "
                      f"{strata} strata by history count, each problem a separate oracle run (setup + cycles of "
                      f"point source and OpenMP gen loop on {threads} threads); batch time = sum over strata of "
                      f"mean time per problem x problems",
            "strata": per_stratum}


def batched_section(a, local):
    """The uneven batch: batched form vs the plain forms, tally error vs all-FP64, CPU baseline and
    serving."""
    import numpy as np
    from scone_gb300 import abi, gpu, problems, serve
    out = {"workload": f"batched_uneven_{a.batch_problems}", "precision": "mixed", "transport": "DT"}
    batch = problems.batched_uneven(n_problems=a.batch_problems)
    total = int(sum(pop * c for _, pop, c, _ in batch))
    out["histories_per_step"] = total
    out["problems"] = len(batch)

    def load(prec):
        B = gpu.BatchGPU(precision=prec, transport=abi.TRANSPORT_DT, device=local, max_problems=2 * len(batch),
                         arena_bytes=(1 << 30) if a.profile else (4 << 30), max_work_items=1 << 21)
        return B, [B.add(p, pop, c, m) for p, pop, c, m in batch]

    B, slots = load(abi.PREC_MIXED)
    # autotuner on a stratified sample (every 8th problem), then the full batch
    t0 = time.perf_counter()
    out["tuning"] = B.tuning() if a.no_autotune else B.autotune(slots[::8])
    out["autotune_s"] = time.perf_counter() - t0
    B.run(slots)                                                       # warm-up
    for s in slots:
        B.clear_tally(s)
    steps = max(1, min(a.steps, 3))
    ms, walls = [], []
    ev = 0
    for _ in range(steps):
        w0 = time.perf_counter()
        st = B.run(slots)
        walls.append(time.perf_counter() - w0)
        ms.append(st.run_ms)
        ev = st.n_events
    mean_ms = sum(ms) / len(ms)
    out["value"] = total / (mean_ms / 1e3)
    out["unit"] = "histories/s"
    out["wall_value"] = total / (sum(walls) / len(walls))
    out["events_per_s"] = ev / (mean_ms / 1e3)
    out["ms_per_step"] = mean_ms
    out["gpu_launches_per_step"] = 2
    # one clean run for the tally comparison with the FP64 form (the timed runs accumulated)
    for s in slots:
        B.clear_tally(s)
    B.run(slots)
    mixed_bins = [B.bins(s) for s in slots]
    # e2e: the public call plus the read-back of every problem's bins to the host
    t0 = time.perf_counter()
    B.run(slots)
    d2h = 0
    for s in slots:
        d2h += B.bins(s).nbytes
    we = time.perf_counter() - t0
    out["e2e"] = {"value": total / we, "unit": "histories/s", "h2d_bytes_per_step": 16 * st.n_items + 4 * len(slots),
                  "d2h_bytes_per_step": d2h}
    # roofline of the batched kernel (same per-event bytes as the single-problem history loop)
    peak, kind = measured_peaks()
    ach = ev * BYTES_PER_EVENT_MIXED / (mean_ms / 1e3) / 1e9
    bpe_dram = committed_traffic("k_batch_uneven")
    out["roofline"] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                       "peak_source": kind, "kernel": "k_batch (batched history loop)",
                       "traffic": bpe_dram * ev if bpe_dram else None, "bytes_per_event": BYTES_PER_EVENT_MIXED,
                       "events_per_launch": ev, "launch_ms": mean_ms,
                       "launch_ms_spans": "the run graph (work-list copy, counter reset, k_batch, k_batch_close), "
                                          "CUDA events on the batch stream; k_batch is ~100 % of it"}
    comp = committed_compute("k_batch_uneven")
    if comp:
        out["roofline"]["compute"] = comp
    if not a.no_plain:
      try:
        # the event form's queue thresholds tuned on a sample (every 64th problem), as the batch's
        t0 = time.perf_counter()
        out["plain_event_tuning"] = B.autotune_plain(slots[::64])
        out["plain_autotune_s"] = time.perf_counter() - t0
        for name, form in (("plain_event", abi.FORM_EVENT), ("plain_history", abi.FORM_HISTORY)):
            B.run_plain(slots[:4], form=form)                          # warm-up (work handle, modules)
            for s in slots:
                B.clear_tally(s)
            t0 = time.perf_counter()
            st = B.run_plain(slots, form=form)
            w = time.perf_counter() - t0
            out[name] = {"value": total / w, "unit": "histories/s", "wall_s": w, "kernels": int(st.n_kernels),
                         "device_value": total / (st.run_ms / 1e3), "run_ms": st.run_ms,
                         "transport_kernel_ms": st.kernel_ms}
        # like with like: wall clock against wall clock, device time against device time
        for name in ("plain_event", "plain_history"):
            out[f"speedup_vs_{name}"] = {"wall": out["wall_value"] / out[name]["value"],
                                         "device": out["value"] / out[name]["device_value"]}
      except Exception as e:
        out["plain_error"] = repr(e)
    B64 = s64 = None
    if not a.no_fp64_batch:
      try:
        B64, s64 = load(abi.PREC_FP64)
        t0 = time.perf_counter()
        st = B64.run(s64)
        out["fp64"] = {"value": total / (st.run_ms / 1e3), "unit": "histories/s", "ms_per_step": st.run_ms}
        ratios, zs = [], []
        for mb, s in zip(mixed_bins, s64):
            fb = B64.bins(s)
            n = 10
            m1, m2 = fb[:, 1] / n, mb[:, 1] / n
            v1 = np.maximum(fb[:, 2] / n - m1 ** 2, 0) / (n - 1)
            v2 = np.maximum(mb[:, 2] / n - m2 ** 2, 0) / (n - 1)
            ok = (v1 > 0) & (v2 > 0) & (m1 > 0)
            ratios += (np.sqrt(v2[ok]) / m2[ok] / (np.sqrt(v1[ok]) / m1[ok])).tolist()
            zs += ((m2[ok] - m1[ok]) / np.sqrt(v1[ok] + v2[ok])).tolist()
        r = np.abs(np.array(ratios) - 1.0)
        out["tally_rel_error_vs_fp64"] = {"bins": len(ratios), "median_abs_dev": float(np.median(r)),
                                          "p99_abs_dev": float(np.percentile(r, 99)),
                                          "frac_within_10pct": float(np.mean(r < 0.10)),
                                          "max_abs_z": float(np.max(np.abs(zs)))}
      except Exception as e:
        out["fp64_error"] = repr(e)
    if not a.no_cpu_baseline:
      try:
        out["cpu_baseline"] = batch_cpu_baseline(batch, os.cpu_count() or 1)
        out["speedup_vs_cpu"] = out["value"] / out["cpu_baseline"]["value"]
      except Exception as e:
        out["cpu_baseline"] = {"value": None, "sample": f"failed: {e}"}
    if not a.no_serve and a.serve_seconds > 0:
      try:
        templates = [(pop, c) for _, pop, c, _ in batch]
        mean_hist = float(np.mean([pop * c for pop, c in templates]))
        lat = problems.lattice_17x17_7g()
        res = {}
        cap = out["value"]
        tuning = out["tuning"]
        B.close()
        B = None
        for name, rate, efrac, secs in (("mix_2000rps_5pct_eigen", 2000.0, 0.05, a.serve_seconds),
                                        ("half_capacity", 0.5 * cap / mean_hist, 0.0, min(a.serve_seconds, 20.0))):
            Bs, cat = load(abi.PREC_MIXED)
            Bs.set_tuning(**tuning)
            pool = serve.EigenPool(lat, 2, abi.PREC_MIXED, abi.TRANSPORT_DT, 100000) if efrac > 0 else None
            S = serve.SolveServer(Bs, cat, wave_histories=a.wave_histories, item_histories=a.serve_item, eigen=pool,
                                  eigen_queue_max=4 if efrac > 0 else None,
                                  defer_backlog=2 * a.wave_histories if efrac > 0 else None)
            offered = rate * ((1 - efrac) * mean_hist + efrac * 100000 * 60)
            qlog = []
            done, wall, n = serve.poisson_run(S, templates, rate, secs, seed=7, eigen_fraction=efrac,
                                              drain=(efrac == 0), max_drain_s=30.0, queue_log=qlog)
            S.stop()
            sh, se = Bs.serve_counts()
            summ = serve.latency_summary(done, wall, offered)
            summ["fixed_source_events_per_s"] = se / wall
            summ["roofline_frac"] = se * BYTES_PER_EVENT_MIXED / wall / 1e9 / measured_peaks()[0]
            summ.update({"arrival_rate": rate, "arrived": n, "eigen_fraction": efrac, "seconds": secs,
                         "eigen_completed": sum(1 for r in done if r.kind == "eigen" and r.status == "done"),
                         "waves": Bs.serve_status()[2], "queues": serve.queue_growth(qlog)})
            if efrac > 0:
                summ["eigen_policy"] = {"pool": 2, "queue_max": 4, "defer_backlog_histories": 2 * a.wave_histories,
                                        "deferred_turns": S.deferred_turns, "shed": S.shed,
                                        "rule": "at most 2 eigenvalue requests run; an arrival finding 4 waiting is "
                                                "shed; eigenvalue cycles wait while fixed-source requests wait for "
                                                "memory or more than 2 waves of histories are queued"}
            # per-request tally error against the all-FP64 form: a sample of completed fixed-source
            # requests re-run as FP64 instances with the same sizes and seeds
            if B64 is not None:
                fixed = [r for r in done if r.kind == "fixed" and r.bins is not None]
                rng = np.random.default_rng(11)
                pick = [fixed[i] for i in rng.choice(len(fixed), size=min(256, len(fixed)), replace=False)]
                inst = [B64.instance(s64[r.template], r.pop, r.cycles, r.master) for r in pick]
                B64.run(inst)
                per = []
                for r, sl in zip(pick, inst):
                    d = tally_deviation(B64.bins(sl), r.bins, r.cycles)
                    if d["bins"]:
                        per.append((d["max_abs_z"], d["frac_rel_err_within_10pct"], d["rel_err_ratio_median_abs_dev"]))
                    B64.remove(sl)
                if per:
                    per = np.array(per)
                    summ["per_request_tally_vs_fp64"] = {
                        "requests": int(per.shape[0]), "max_abs_z_median": float(np.median(per[:, 0])),
                        "max_abs_z_p99": float(np.percentile(per[:, 0], 99)),
                        "frac_bins_rel_err_within_10pct_mean": float(per[:, 1].mean()),
                        "frac_requests_all_bins_within_10pct": float(np.mean(per[:, 1] == 1.0)),
                        "rel_err_ratio_median_abs_dev_median": float(np.median(per[:, 2])),
                        "how": "sampled completed requests re-run as all-FP64 batch instances (same template, "
                               "population, cycles, seed); per bin z and relative-error ratio"}
            res[name] = summ
            if pool:
                for t_, _ in pool.free:
                    t_.close()
            Bs.close()
        out["serving"] = res
      except Exception as e:
        out["serving_error"] = repr(e)
    if B64 is not None:
        B64.close()
    if B is not None:
        B.close()
    return out


def profile_ce_cycle(local, pop=200_000):
    """For ncu captures: two fixed-source cycles of the continuous-energy 3-layer slab (mixed form,
    delta tracking), the second one the captured launch."""
    from scone_gb300 import abi, gpu, problems
    p = problems.ce_slab_3layer()
    t = gpu.TransportOperatorGPU(p, precision=abi.PREC_MIXED, transport=abi.TRANSPORT_DT, max_bank=pop + 4096,
                                 device=local, form=abi.FORM_HISTORY)
    adm = t.upload_tally(p.tallies["current"])
    m = SEED
    for _ in range(2):
        m, _st = t.fixed_source_cycle(adm, pop, m)
    t.close()


def committed_compute(kernel):
    """Compute-side counters of `kernel` from its committed ncu capture (profiles/compute.json)."""
    p = os.path.join(ROOT, "profiles", "compute.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f).get(kernel)
    return None


def main():
    a = args_()
    rank, world, local = dist_env()
    from scone_gb300 import abi, problems
    p = problems.lattice_17x17_7g()
    if a.impl == "reference":
        line = reference_arm(a, p)
        if line is not None:
            print(json.dumps(line), flush=True)
        return

    import torch
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist
    from scone_gb300 import gpu

    prec = abi.PREC_MIXED if a.precision == "mixed" else abi.PREC_FP64
    tr = transport_code(a)
    cap = int(2.5 * a.pop) + 4096
    form = abi.FORM_EVENT if a.form == "event" else abi.FORM_HISTORY
    t = gpu.TransportOperatorGPU(p, precision=prec, transport=tr, max_bank=cap, device=local, form=form)
    inact, ia, act, aa = lattice_setup(t, p)
    # replicas: rank r uses the master stream strided by r * pop (SCONE's getOffset sharding)
    master0 = gpu.rng_skip(SEED, 152917 * rank * a.pop)
    t.eigen_init(a.pop, master0)
    warm = max(3, a.warmup)
    for _ in range(warm):
        t.eigen_cycle(inact, ia)

    sampler = ClockSampler(local)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)
    wall0 = time.perf_counter()
    cyc_ms = tr_ms = 0.0
    events = launches = hist = 0
    ks = []
    for _ in range(a.steps):
        st = t.eigen_cycle(act, aa)
        cyc_ms += st.cycle_ms
        tr_ms += st.transport_ms
        events += st.n_events
        launches += st.n_kernels
        hist += st.n_histories
        ks.append(st.k_new)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if pg:
        pg.barrier()
    clocks = sampler.stop()

    # e2e: the same cycle through the C ABI with host banks (sg_eigen_cycle_bank: what a Fortran
    # eigenPhysicsPackage that keeps its dungeons in host memory calls once per cycle), starting from
    # the converged bank and pRNG of the run above; the bank is page-locked host memory that the
    # kernels read in place, and the normalised next bank is copied back every step
    e2e = None
    e2e_gen = None
    if not a.no_e2e:
        import ctypes as C
        bank, pop = t.eigen_bank(a.pop)
        master, k = t.eigen_state()
        b_in, b_out = pinned_bank(bank, pop, pop), pinned_bank(None, 0, pop)
        e_act = t.upload_tally(p.tallies["mesh"])
        e_aa = t.upload_tally([abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
        t.attach_tally(e_act, e_aa)
        k_end = k
        for _ in range(2):                                             # warm-up
            master, k, _st = t.eigen_cycle_bank(e_act, e_aa, b_in, pop, master, k, k_end, b_out)
            k_end = k
            b_in, b_out = b_out, b_in
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        e_tr = e_cyc = 0.0
        for _ in range(a.steps):
            master, k, _st = t.eigen_cycle_bank(e_act, e_aa, b_in, pop, master, k, k_end, b_out)
            e_tr += _st.transport_ms
            e_cyc += _st.cycle_ms
            k_end = k
            b_in, b_out = b_out, b_in
        torch.cuda.synchronize()
        we = time.perf_counter() - w0
        e2e = {"value": a.steps * pop / we, "unit": "histories/s",
               "h2d_bytes_per_step": pop * (24 + 24 + 8 + 4 + 8),
               "d2h_bytes_per_step": pop * (24 + 24 + 8 + 4 + 8 + 4), "ms_per_step": 1e3 * we / a.steps,
               "call": "sg_eigen_cycle_bank (one whole cycle per call, host dungeons)",
               "h2d": "page-locked host bank read in place by the kernels across the host link (no staging copy)",
               "d2h": "normalised next-cycle bank, cudaMemcpyAsync after the cycle",
               "transport_kernel_ms_per_step": e_tr / a.steps, "call_device_ms_per_step": e_cyc / a.steps}
        e2e["link_d2h_gbps"] = link_d2h_gbps(e2e["d2h_bytes_per_step"])
        e2e["d2h_ms_at_link_rate"] = e2e["d2h_bytes_per_step"] / (e2e["link_d2h_gbps"] * 1e6)
        # the gen loop alone through sg_transport_bank (a shim that keeps normSize_Repr in Fortran)
        nxt_cap = cap
        b_next = pinned_bank(None, 0, nxt_cap)
        adm_e2e = t.upload_tally(p.tallies["mesh"] + [abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
        for w_ in range(2):
            st = abi.CycleStats()
            t._check(t.L.sg_transport_bank(t.h, adm_e2e, C.byref(b_in.struct), pop, C.c_uint64(55 + w_), 1.0,
                                           C.byref(b_next.struct), nxt_cap, C.byref(st)))
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        d2h = 0
        for s_ in range(a.steps):
            t.tally_cycle_start(adm_e2e, float(pop))
            st = abi.CycleStats()
            t._check(t.L.sg_transport_bank(t.h, adm_e2e, C.byref(b_in.struct), pop, C.c_uint64(1000 + s_), ks[-1],
                                           C.byref(b_next.struct), nxt_cap, C.byref(st)))
            t.tally_cycle_end(adm_e2e, float(st.n_next), ks[-1])
            d2h += st.n_next * (24 + 24 + 8 + 4 + 8 + 4)
        torch.cuda.synchronize()
        we = time.perf_counter() - w0
        e2e_gen = {"value": a.steps * pop / we, "unit": "histories/s", "h2d_bytes_per_step": pop * 68,
                   "d2h_bytes_per_step": int(d2h / a.steps), "ms_per_step": 1e3 * we / a.steps,
                   "call": "sg_tally_cycle_start + sg_transport_bank + sg_tally_cycle_end (gen loop and site "
                           "order only; normSize_Repr left to the caller)"}

    # the other transport operator on the lattice workload (surface tracking vs delta tracking), same K steps
    alt = None
    if not a.no_alt and world == 1:
        tr2 = abi.TRANSPORT_ST if tr == abi.TRANSPORT_DT else abi.TRANSPORT_DT
        t2 = gpu.TransportOperatorGPU(p, precision=prec, transport=tr2, max_bank=cap, device=local, form=form)
        i2, ia2, a2, aa2 = lattice_setup(t2, p)
        t2.eigen_init(a.pop, master0)
        for _ in range(warm):
            t2.eigen_cycle(i2, ia2)
        c2 = e2 = h2 = 0.0
        k2 = None
        for _ in range(a.steps):
            st = t2.eigen_cycle(a2, aa2)
            c2 += st.cycle_ms
            e2 += st.n_events
            h2 += st.n_histories
            k2 = st.k_new
        alt = {"transport": "ST" if tr2 == abi.TRANSPORT_ST else "DT", "value": h2 / (c2 / 1e3),
               "unit": "histories/s", "events_per_s": e2 / (c2 / 1e3), "ms_per_step": c2 / a.steps, "k_eff": k2}
        t2.close()

    # the lattice in the other execution form (the event-based plain form against the history loop),
    # same K steps: the measurement behind keeping the history loop as the fast form
    other_form = None
    if not a.no_alt and world == 1:
        f2 = abi.FORM_HISTORY if form == abi.FORM_EVENT else abi.FORM_EVENT
        t3 = gpu.TransportOperatorGPU(p, precision=prec, transport=tr, max_bank=cap, device=local, form=f2)
        i3, ia3, a3, aa3 = lattice_setup(t3, p)
        t3.eigen_init(a.pop, master0)
        for _ in range(warm):
            t3.eigen_cycle(i3, ia3)
        c3 = tk3 = h3 = 0.0
        n3 = 0
        for _ in range(a.steps):
            st = t3.eigen_cycle(a3, aa3)
            c3 += st.cycle_ms
            tk3 += st.transport_ms
            h3 += st.n_histories
            n3 += st.n_kernels
        other_form = {"form": "event" if f2 == abi.FORM_EVENT else "history", "value": h3 / (c3 / 1e3),
                      "unit": "histories/s", "ms_per_step": c3 / a.steps, "transport_ms_per_step": tk3 / a.steps,
                      "kernels_per_step": n3 / a.steps}
        t3.close()

    # max over ranks of the device time; histories summed over ranks
    sec = cyc_ms / 1e3
    if pg:
        tt = torch.tensor([sec, float(hist), float(events)], device="cuda", dtype=torch.float64)
        mx = tt.clone()
        pg.all_reduce(mx[:1], op=pg.ReduceOp.MAX)
        pg.all_reduce(tt[1:], op=pg.ReduceOp.SUM)
        sec, hist, events = float(mx[0]), int(tt[1]), int(tt[2])
        if e2e:
            te = torch.tensor([e2e["value"]], device="cuda", dtype=torch.float64)
            pg.all_reduce(te, op=pg.ReduceOp.SUM)
            e2e["value"] = float(te[0])
    if rank != 0:
        if pg:
            pg.destroy_process_group()
        return

    bpe = BYTES_PER_EVENT_MIXED if prec == abi.PREC_MIXED else BYTES_PER_EVENT_FP64
    peak, peak_kind = measured_peaks()
    ev_per_launch = events / (a.steps * world)
    launch_ms = tr_ms / a.steps
    achieved = ev_per_launch * bpe / (launch_ms / 1e3) / 1e9
    bpe_dram = committed_traffic("k_transport_lattice")
    traffic = bpe_dram * ev_per_launch if bpe_dram else None
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "peak_source": peak_kind, "kernel": ("event loop: k_ev_start + k_ev_transit + k_ev_collide + k_ev_transit<tail>"
                       if a.form == "event" else "k_transport (history loop)"),
            "bytes_per_event": bpe, "events_per_launch": ev_per_launch, "launch_ms": launch_ms,
            "launch_ms_spans": ("the gen loop's event kernels (start, transit and collision rounds, tail) between "
                                "CUDA events on the library's stream" if a.form == "event" else
                                "the history-loop kernel alone: CUDA events recorded on the library's stream "
                                "directly before and after its one launch per cycle (an active cycle, with the "
                                "mesh tally)")}
    comp = committed_compute("k_transport_lattice")
    if comp:
        roof["compute"] = comp

    cpu = None
    if not a.no_cpu_baseline:
        try:
            threads = os.cpu_count() or 1
            cpu_pop = a.pop
            secs, evs, n = cpu_eigen_cycles(p, cpu_pop, tr, threads, 3, target_s=10.0)
            cpu = {"value": len(secs) * n / sum(secs), "unit": "histories/s", "cores": threads, "kind": "port",
                   "sample": f"3 inactive + {len(secs)} timed active eigenvalue cycles of {n} particles "
                             f"({sum(secs):.1f} s), OpenMP over histories: the code --impl reference times",
                   "events_per_s": sum(evs) / sum(secs)}
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "histories/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {e}"}

    configs = None
    if not a.no_configs and world == 1:
        try:
            configs = configs_section(a, local)
        except Exception as e:
            configs = {"error": repr(e)}
        try:
            configs["lattice_k_vs_fp64"] = lattice_k_section(a, local)
        except Exception as e:
            configs["lattice_k_error"] = repr(e)
    if a.profile and world == 1:
        profile_ce_cycle(local)
    batched = None
    if not a.no_batch and world == 1:
        try:
            batched = batched_section(a, local)
        except Exception as e:  # reported, never silently replaced by anything else
            batched = {"error": repr(e)}

    line = {
        "metric": "histories/s", "value": hist / sec, "unit": "histories/s", "n_gpus": world,
        "steps": a.steps, "warmup": warm, "ms_per_step": 1e3 * sec / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if prec == abi.PREC_MIXED else "f64",
        "data": "synthetic", "precision": a.precision, "form": a.form,
        "config": workload_config(a, world),
        "events_per_s": events / sec, "k_eff": ks[-1], "wall_ms_per_step": 1e3 * wall / a.steps,
        "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
        "e2e_gen_loop_only": e2e_gen, "clocks": clocks,
        "other_transport": alt, "other_form": other_form, "batched": batched, "other_configs": configs,
    }
    print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
