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
    return ap.parse_args()


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


def committed_traffic():
    p = os.path.join(ROOT, "profiles", "transport_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
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

    # the other transport operator of config 1 ("surface tracking vs delta tracking"), same K steps
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
    tr_info = committed_traffic()
    traffic = None
    if tr_info and tr_info.get("bytes_per_event"):
        traffic = tr_info["bytes_per_event"] * ev_per_launch
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
        "other_transport": alt,
    }
    print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
