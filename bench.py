#!/usr/bin/env python3
"""Benchmark of the SCONE particle-tracking cycle on GB300.

Workload: the 17x17 pin-lattice k-eigenvalue problem (7 groups, seeded synthetic XS, pitch 1.26 cm,
pin radius 0.54 cm, reflective box), 1e6 particles per cycle, surface tracking, FP32 XS/distances
with FP64 positions and tally sums.  One step = one active eigenvalue cycle: the gen loop over the
bank, fission-site ordering, tally cycle end (17x17x7 mesh flux + implicit k), normSize_Repr and
k feedback, all resident on the device.

  value  histories/s of the device-resident cycle (CUDA events on the library's stream)
  e2e    histories/s through the C ABI with host banks (sg_transport_bank + tally cycle calls),
         host->device bank copy and device->host fission bank copy inside every step
  roofline  the history-loop kernel: algorithmic bytes (128 B per event, mixed form) / kernel time
  cpu_baseline  the CPU restatement of SCONE (oracle/) on the host cores, bounded sample

Beside the lattice line, the same JSON line carries the uneven batch (4096 independent fixed-source
problems of 1-16 groups, spheres and multi-slabs, 1e3-1e6 histories each, 5.9e8 histories in all):

  batched   histories/s of the batched form (every cycle of every problem in one persistent launch,
            one CUDA graph), mixed precision, delta tracking, launch shape from the autotuner
  plain     histories/s of the plain form over the same batch: one problem per launch sequence
            (sg_fixed_source_cycle per cycle), event-based and history-loop kernels
  tally error  per-bin relative errors of the batched mixed form against the all-FP64 batched form
  serving   Poisson arrivals of requests drawn from the batch (plus 5 % lattice eigenvalue
            requests), continuous batching: p50/p99 latency, achieved and offered histories/s

`--impl reference` times SCONE's algorithm on the host cores instead (the oracle restatement: SCONE
itself is Fortran and cannot be built here), on the same workload and metric.
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
    ap.add_argument("--pop", type=int, default=1_000_000)
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
    ap.add_argument("--serve-seconds", type=float, default=15.0)
    ap.add_argument("--wave-histories", type=int, default=1 << 23, help="histories per serving wave")
    ap.add_argument("--serve-item", type=int, default=256, help="histories per work item while serving")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shape of the batch")
    ap.add_argument("--no-configs", action="store_true", help="skip the infinite-medium and CE-slab lines")
    a = ap.parse_args()
    if a.profile:   # a short run for ncu: lattice cycles and one small batch, nothing else
        a.no_cpu_baseline = a.no_e2e = a.no_alt = a.no_plain = a.no_fp64_batch = a.no_serve = True
        a.no_autotune = a.no_configs = True
        a.batch_problems = min(a.batch_problems, 256)
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


def cpu_rate(p, pop_bank, threads, target_s=10.0, max_hist=2_000_000, transport=None):
    """Histories/s of the oracle's OpenMP gen loop on the host cores over a bounded sample: the
    bank is transported repeatedly (fresh RNG streams) until about target_s seconds have passed."""
    from oracle import oracle
    from scone_gb300 import abi
    o = oracle.Oracle(p, transport=abi.TRANSPORT_ST if transport is None else transport)
    adm = o.upload_tally(p.tallies["mesh"] + [abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
    n = min(max_hist, len(pop_bank["wgt"]))
    bank = abi.HostBank(n, {k: v[:n] for k, v in pop_bank.items()})
    hist = ev = 0
    t0 = time.perf_counter()
    rep = 0
    while True:
        nh, e = o.timed_gen_loop(adm, bank, 12345 + 7919 * rep, 1.0, threads)
        hist += nh
        ev += e
        rep += 1
        dt = time.perf_counter() - t0
        if dt >= target_s:
            break
    return hist / dt, ev / dt, hist, dt


def host_bank_dict(b, n):
    return {k: b[k][:n].copy() for k in ("wgt", "r", "dir", "G", "time", "brood_id")}


def reference_arm(a, p):
    """SCONE's algorithm on the host cores (oracle restatement), same workload and metric."""
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    from oracle import oracle
    from scone_gb300 import abi
    threads = os.cpu_count() or 1
    tr = {"st": abi.TRANSPORT_ST, "dt": abi.TRANSPORT_DT, "st-nocache": abi.TRANSPORT_ST_NOCACHE}[a.transport]
    o = oracle.Oracle(p, transport=tr)
    o.eigen_init(a.pop, SEED)
    bank, pop = o.eigen_bank(a.pop)
    bd = host_bank_dict(bank, pop)
    # one step = a bounded sample of one cycle's gen loop (the bank of `pop` histories)
    n = pop
    adm = o.upload_tally(p.tallies["mesh"] + [abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
    hb = abi.HostBank(n, {k: v[:n] for k, v in bd.items()})
    for _ in range(a.warmup):
        o.timed_gen_loop(adm, hb, 777, 1.0, threads)
    tot, ev = 0.0, 0
    for s in range(a.steps):
        t0 = time.perf_counter()
        nh, e = o.timed_gen_loop(adm, hb, 1000 + s, 1.0, threads)
        tot += time.perf_counter() - t0
        ev += e
    value = a.steps * n / tot
    line = {
        "impl": "reference", "metric": "histories/s", "value": value, "unit": "histories/s",
        "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * tot / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "events_per_s": ev / tot,
        "config": {"workload": "lattice_17x17_7g_eigen", "particles_per_cycle": n, "groups": 7,
                   "lattice": "17x17 pins r=0.54 pitch=1.26", "transport": a.transport.upper(),
                   "reference": "C++ restatement of SCONE's algorithm (oracle/); SCONE is Fortran and no "
                                "Fortran compiler exists here"},
        "cpu_baseline": {"value": value, "unit": "histories/s", "cores": threads, "kind": "port",
                         "sample": f"each step: the gen loop over the {n}-particle initial fission bank, "
                                   f"OpenMP over histories on {threads} threads"},
        "e2e": {"value": value, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


def lattice_k_section(a, local):
    """Lattice k of the mixed form against the all-FP64 form: the same inactive and active cycles
    (1e5 particles, 10 + 20 cycles, delta tracking) in both; z = difference over the combined sigma."""
    from scone_gb300 import abi, gpu, problems
    p = problems.lattice_17x17_7g()
    res = {}
    for name, prec in (("mixed", abi.PREC_MIXED), ("fp64", abi.PREC_FP64)):
        t = gpu.TransportOperatorGPU(p, precision=prec, transport=abi.TRANSPORT_DT, max_bank=300000, device=local,
                                     form=abi.FORM_HISTORY)
        inact, ia, act, aa = lattice_setup(t, p)
        t.eigen_init(100000, SEED)
        for _ in range(10):
            t.eigen_cycle(inact, ia)
        for _ in range(20):
            t.eigen_cycle(act, aa)
        res[name] = t.keff(aa)
        t.close()
    (km, sm), (kd, sd) = res["mixed"], res["fp64"]
    return {"k_mixed": km, "sigma_mixed": sm, "k_fp64": kd, "sigma_fp64": sd,
            "z": (km - kd) / (sm * sm + sd * sd) ** 0.5, "cycles": "10 inactive + 20 active, 1e5 particles"}


def configs_section(a, local):
    """The other two workloads, each through sg_fixed_source_cycle on its own handle (device-resident
    source, gen loop and batch close) and through the oracle on the host cores:
    infinite homogeneous medium, 2 groups, 1e5 histories; continuous-energy 3-layer slab, 1e7
    histories (10 cycles of 1e6), FP32 tables with FP64 energy and position."""
    from oracle import oracle
    from scone_gb300 import abi, gpu, problems
    threads = os.cpu_count() or 1
    out = {}
    cases = [("infinite_medium_2g", problems.infinite_medium_2g(), "flux", 100000, 1, abi.TRANSPORT_ST),
             ("ce_slab_3layer", problems.ce_slab_3layer(), "current", 1000000, 10, abi.TRANSPORT_DT)]
    for name, p, tally, pop, cycles, tr in cases:
        res = {"histories": pop * cycles, "transport": "ST" if tr == abi.TRANSPORT_ST else "DT"}
        for prec_name, prec in (("mixed", abi.PREC_MIXED), ("fp64", abi.PREC_FP64)):
            t = gpu.TransportOperatorGPU(p, precision=prec, transport=tr, max_bank=pop + 4096, device=local,
                                         form=abi.FORM_HISTORY)
            adm = t.upload_tally(p.tallies[tally])
            m = SEED
            t.fixed_source_cycle(adm, min(pop, 10000), m)                # warm-up
            ms = ev = 0.0
            for _ in range(cycles):
                m, st = t.fixed_source_cycle(adm, pop, m)
                ms += st.cycle_ms
                ev += st.n_events
            res[prec_name] = {"value": pop * cycles / (ms / 1e3), "unit": "histories/s",
                              "events_per_s": ev / (ms / 1e3), "ms": ms}
            t.close()
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


def batched_section(a, local):
    """The uneven batch: batched form vs the plain forms, tally error vs all-FP64, and serving."""
    import numpy as np
    from scone_gb300 import abi, gpu, problems, serve
    out = {"workload": f"batched_uneven_{a.batch_problems}", "precision": "mixed", "transport": "DT"}
    batch = problems.batched_uneven(n_problems=a.batch_problems)
    total = int(sum(pop * c for _, pop, c, _ in batch))
    out["histories_per_step"] = total
    out["problems"] = len(batch)

    def load(prec):
        B = gpu.BatchGPU(precision=prec, transport=abi.TRANSPORT_DT, device=local, max_problems=2 * len(batch),
                         arena_bytes=4 << 30, max_work_items=1 << 21)
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
    ms = []
    ev = 0
    for _ in range(steps):
        st = B.run(slots)
        ms.append(st.run_ms)
        ev = st.n_events
    mean_ms = sum(ms) / len(ms)
    out["value"] = total / (mean_ms / 1e3)
    out["unit"] = "histories/s"
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
                       "events_per_launch": ev, "launch_ms": mean_ms}
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
                         "transport_kernel_ms": st.kernel_ms}
        out["speedup_vs_plain_event"] = out["value"] / out["plain_event"]["value"]
        out["speedup_vs_plain_history"] = out["value"] / out["plain_history"]["value"]
      except Exception as e:
        out["plain_error"] = repr(e)
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
        B64.close()
      except Exception as e:
        out["fp64_error"] = repr(e)
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
        for name, rate, efrac in (("mix_2000rps_5pct_eigen", 2000.0, 0.05),
                                  ("half_capacity", 0.5 * cap / mean_hist, 0.0)):
            Bs, cat = load(abi.PREC_MIXED)
            Bs.set_tuning(**tuning)
            pool = serve.EigenPool(lat, 4, abi.PREC_MIXED, abi.TRANSPORT_DT, 100000) if efrac > 0 else None
            S = serve.SolveServer(Bs, cat, wave_histories=a.wave_histories, item_histories=a.serve_item, eigen=pool)
            offered = rate * ((1 - efrac) * mean_hist + efrac * 100000 * 60)
            done, wall, n = serve.poisson_run(S, templates, rate, a.serve_seconds, seed=7, eigen_fraction=efrac,
                                              drain=(efrac == 0), max_drain_s=30.0)
            S.stop()
            sh, se = Bs.serve_counts()
            summ = serve.latency_summary(done, wall, offered)
            summ["fixed_source_events_per_s"] = se / wall
            summ["roofline_frac"] = se * BYTES_PER_EVENT_MIXED / wall / 1e9 / measured_peaks()[0]
            summ.update({"arrival_rate": rate, "arrived": n, "eigen_fraction": efrac,
                         "eigen_completed": sum(1 for r in done if r.kind == "eigen"),
                         "waves": Bs.serve_status()[2]})
            res[name] = summ
            if pool:
                for t, _ in pool.free:
                    t.close()
            Bs.close()
        out["serving"] = res
      except Exception as e:
        out["serving_error"] = repr(e)
    if B is not None:
        B.close()
    return out


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
    tr = {"st": abi.TRANSPORT_ST, "dt": abi.TRANSPORT_DT, "st-nocache": abi.TRANSPORT_ST_NOCACHE}[a.transport]
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

    # e2e: the same cycles through the host-bank C ABI (what a Fortran physicsPackage calls)
    e2e = None
    if not a.no_e2e:
        bank, pop = t.eigen_bank(a.pop)
        pin = {k: torch.from_numpy(v).pin_memory() for k, v in host_bank_dict(bank, pop).items()}
        hb = abi.HostBank(pop, {k: v.numpy() for k, v in pin.items()})
        nxt_cap = cap
        pin_next = {k: torch.empty((nxt_cap, 3) if k in ("r", "dir") else (nxt_cap,),
                                   dtype=torch.float64 if k in ("wgt", "r", "dir", "time") else torch.int32).pin_memory()
                    for k in ("wgt", "r", "dir", "G", "time", "brood_id")}
        nb = abi.HostBank(nxt_cap, {k: v.numpy() for k, v in pin_next.items()})
        import ctypes as C
        adm_e2e = t.upload_tally(p.tallies["mesh"] + [abi.clerk(abi.CLERK_KEFF_IMPLICIT)])
        for w_ in range(2):
            st = abi.CycleStats()
            t._check(t.L.sg_transport_bank(t.h, adm_e2e, C.byref(hb.struct), pop, C.c_uint64(55 + w_), 1.0,
                                           C.byref(nb.struct), nxt_cap, C.byref(st)))
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        d2h = 0
        for s in range(a.steps):
            t.tally_cycle_start(adm_e2e, float(pop))
            st = abi.CycleStats()
            t._check(t.L.sg_transport_bank(t.h, adm_e2e, C.byref(hb.struct), pop, C.c_uint64(1000 + s), ks[-1],
                                           C.byref(nb.struct), nxt_cap, C.byref(st)))
            t.tally_cycle_end(adm_e2e, float(st.n_next), ks[-1])
            d2h += st.n_next * (24 + 24 + 8 + 4 + 8 + 4)
        torch.cuda.synchronize()
        we = time.perf_counter() - w0
        e2e = {"value": a.steps * pop / we, "unit": "histories/s",
               "h2d_bytes_per_step": pop * (24 + 24 + 8 + 4 + 8),
               "d2h_bytes_per_step": int(d2h / a.steps), "ms_per_step": 1e3 * we / a.steps}

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
            "bytes_per_event": bpe, "events_per_launch": ev_per_launch, "launch_ms": launch_ms}

    cpu = None
    if not a.no_cpu_baseline:
        try:
            bank, pop = t.eigen_bank(min(a.pop, 400000))
            bd = host_bank_dict(bank, min(pop, 400000))
            threads = os.cpu_count() or 1
            rate, erate, n, dt = cpu_rate(p, bd, threads, transport=tr)
            cpu = {"value": rate, "unit": "histories/s", "cores": threads, "kind": "port",
                   "sample": f"{n} histories (lattice bank of {min(pop, 400000)} transported repeatedly), "
                             f"{dt:.1f} s, OpenMP over histories",
                   "events_per_s": erate}
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
        "data": "synthetic",
        "config": {"workload": "lattice_17x17_7g_eigen", "particles_per_cycle": a.pop, "groups": 7,
                   "lattice": "17x17 pins r=0.54 cm pitch=1.26 cm, reflective box", "transport": a.transport.upper(),
                   "precision": a.precision, "form": a.form, "step": "one active eigenvalue cycle (gen loop + site order + "
                   "tally close + normSize_Repr + k feedback)", "tally": "17x17x7 mesh flux + implicit k",
                   "l2": "per-step working set exceeds L2 (bank 72 MB in, ~80 MB sites, 72 MB ordered, 72 MB normalised)",
                   "parallelism": f"replicas{world}"},
        "events_per_s": events / sec, "k_eff": ks[-1], "wall_ms_per_step": 1e3 * wall / a.steps,
        "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
        "other_transport": alt, "batched": batched, "other_configs": configs,
    }
    print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
