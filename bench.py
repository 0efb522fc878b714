"""Benchmark: ray-segments/s of the stochastic energy tracer on one GB300.

Workload (the 50k-triangle multi-room scene): 40 box rooms on an 8 x 5 grid
with shared walls, 1 x 2.1 m door holes and glass panes, 49k primitives after
tessellation; 64 source/listener pairs x 4096 rays x 3 bands, 2000 x 1 ms
bins (2 s), <= 200 bounces, energy floor 1e-6; plus the 512-ray golden-spiral
dome fan for each of the 64 listeners. A step traces all 64 pairs, then the
64 domes on the same stream. Inputs (scene,
jobs) are resident in HBM; the BVH (~3 MB) fits in L2, so L2 is flushed (a
256 MB write) before every timed step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

The near-tie rule (tie_mode 1: lowest surface id among hits within 1e-6
relative t) is on, so the f32 result matches the FP64 oracle.

Beside the headline, the line carries the learned surrogate against the
tracer ("surrogate") and the world early reflections on the same scene
("early": chain discovery and the batched exact solve of every source x chain
pair, with the oracle's solve of a sample timed beside it).

Rank 0 prints one JSON line. `--impl reference` times the CPU restatement of
the reference tracer (the oracle port; the reference itself is Rust and has
no toolchain here) on the host cores, on the same metric.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ray-segments/s on 1 GB300 (% HBM roofline); surrogate vs tracer ms/room at <=5% RT60 err"
UNIT = "ray-segments/s"
N_PAIRS = 64
N_RAYS = 4096
DOME_RAYS = 512
CFG = dict(n_bands=3, n_bins=2000, bin_dt=0.001, max_time=2.0, max_bounces=200, energy_floor=1e-6)
WORKLOAD = "multiroom-40rooms-49k-prims: 64 pairs x 4096 rays x 3 bands, 2000 x 1 ms bins, 200 bounces, " \
           "floor 1e-6, + 64 x 512-ray dome fans"


def traffic():
    """DRAM bytes (read + write) of one trace part, from the ncu capture whose
    summary is committed under profiles/ (None when there is none)."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh).get("trace_multiroom_64x4096", {}).get("dram_bytes")
    return None


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows for n, v in zip(names, r[5:9]) if v.strip().lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def build_case():
    from omg_audio_gb300 import workloads as W
    return W.multiroom(seed=2, n_pairs=N_PAIRS)


def oracle_mesh(case, real="f32"):
    from oracle import oracle as O
    mb = O.MeshBuilder()
    case.recorder.replay(mb, lambda m: O.Material.make(m.absorption, m.scattering, m.transmission))
    return mb.build(real)


def cpu_sample(case, n_pairs, threads, n_rays=N_RAYS, ray_end=None, fans=True):
    """The f32 oracle running the reference's own algorithm: its first-found
    closest hit (tie_mode 0, mesh.rs:505) over its own SAH tree
    (mesh.rs:241-405), in its f32 arithmetic, on pairs [0, n_pairs), then (fans)
    the 512-ray dome fan of each of those pairs' listeners (dome.rs:425-478).
    Returns segments, seconds and the trace's traversal counters."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O
    mesh = oracle_mesh(case)
    P = O.params(tie_mode=0, **CFG)
    pan = [(mn, mx, O.Material.make(m.absorption, m.scattering, m.transmission)) for (mn, mx, m) in case.panels]
    tot = {k: 0 for k in ("segments", "receiver_hits") + O.TRAV_KEYS}
    glass = [g.as_dict() for g in case.glass]
    eyes = [lis for (_, lis) in case.pairs[:n_pairs]] if fans else []
    probes = [O.DomeProbe(mesh, glass, n_fan=DOME_RAYS, nb=3) for _ in range(min(threads, len(eyes)))]
    t0 = time.perf_counter()
    for p in range(n_pairs):
        src, lis = case.pairs[p]
        _, _, st = O.trace_mesh(mesh, src, lis, n_rays, P=P, seed=1000 + p, panels=pan, threads=threads,
                                ray_end=ray_end)
        for k in tot:
            tot[k] += st[k]
    dome_seg = 0
    if eyes:
        # one probe per host thread (ctypes releases the GIL during the call)
        def fan(i):
            pr = probes[i]
            n = 0
            for eye in eyes[i::len(probes)]:
                r = pr.sample(eye, (), n_rays=DOME_RAYS)
                n += r["stats"]["escape_events"] + r["stats"]["through_calls"]
            return n
        with ThreadPoolExecutor(len(probes)) as ex:
            dome_seg = sum(ex.map(fan, range(len(probes))))
    dt = time.perf_counter() - t0
    del probes
    return dict(tot, seconds=dt, dome_segments=dome_seg)


def bytes_per_segment(st, nb=3):
    """B_seg = 32 N_node + 48 N_prim + 4 (NB + 3) h, per segment of the reference's
    ordered traversal over its own tree (mesh.rs:484-541): N_node the DISTINCT
    32-byte node records a closest-hit query reads (the root, plus both children
    of every internal node it processes; a child popped later is the record its
    parent already read), N_prim the 48-byte primitives it tests, h the receiver
    hits (one histogram row of NB + 3 floats each)."""
    s = max(st["segments"], 1)
    n_node, n_prim, h = st["unique_nodes"] / s, st["prim_tests"] / s, st["receiver_hits"] / s
    parts = dict(n_node=n_node, n_prim=n_prim, h=h,
                 per_segment={k: st[k] / s for k in ("queries", "internal_visits", "leaf_visits", "child_boxes",
                                                     "unique_nodes", "node_reads", "prim_tests", "receiver_hits")},
                 formula="32 * unique_nodes + 48 * prim_tests + 4 * (NB + 3) * receiver_hits, per segment; "
                         "unique_nodes = queries + child_boxes")
    return 32.0 * n_node + 48.0 * n_prim + 4.0 * (nb + 3) * h, parts


def max_over_ranks(vals, ws, device="cuda"):
    """Per-value maximum over the ranks (one all_reduce MAX); the values
    themselves on one rank. Every rank runs a whole replica of the workload
    (no data-path collective), so the slowest rank's times set the aggregate."""
    if ws <= 1:
        return [float(v) for v in vals]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in vals], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def aggregate_rate(ws, units_per_rank, ms):
    """Whole-job throughput: every rank processed units_per_rank within ms."""
    return ws * units_per_rank / (ms * 1e-3)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def config_of(case_prims):
    """The workload's config, the same dict in both arms."""
    return {"workload": WORKLOAD, "prims": case_prims, "pairs": N_PAIRS, "rays_per_pair": N_RAYS, "bands": 3,
            "bins": CFG["n_bins"], "dome_fans": N_PAIRS, "dome_rays": DOME_RAYS,
            "l2": "GPU arm: flushed (256 MB write) before every timed step; CPU arm: n/a"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    case = build_case()
    threads = os.cpu_count() or 1
    pairs = max(1, min(N_PAIRS, args.ref_pairs))
    for _ in range(max(0, args.warmup)):
        cpu_sample(case, 1, threads, ray_end=256, fans=False)
    times, segs = [], []
    for _ in range(args.steps):
        st = cpu_sample(case, pairs, threads)
        times.append(st["seconds"])
        segs.append(st["segments"] + st["dome_segments"])
    v = float(np.sum(segs) / np.sum(times))
    sample = (f"{pairs} of {N_PAIRS} pairs x {N_RAYS} rays and their {pairs} dome fans per step, "
              f"{threads} host threads")
    prims = oracle_mesh(case).info()["prims"]
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * float(np.mean(times)), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": config_of(prims),
            "impl": "reference",
            "tie_rule": "first found (the reference's, mesh.rs:505) on the reference's SAH tree",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


FWD_FLOP = 2 * (38 * 256 + 3 * 256 * 256 + 256 * 192)   # one sample through the 38-256x4-192 MLP


def gemm_leg(ctx):
    """CUDA-event time of the tensor-core GEMM at the training shapes (rows x
    out x in), operands resident: TFLOP/s and the fraction of the measured bf16
    peak."""
    import ctypes as C

    from omg_audio_gb300 import _lib
    peak = None
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            peak = float(json.load(fh)["bf16_tflops"])
    out = {}
    for name, (m, n, k, split) in {"forward hidden layer 4096x256x256": (4096, 256, 256, 1),
                                   "forward output layer 4096x192x256": (4096, 192, 256, 1),
                                   "weight gradient 256x256 over 4096 rows (K split 8)": (256, 256, 4096, 8),
                                   "input gradient 4096x256x192": (4096, 256, 192, 1)}.items():
        ms = C.c_float()
        ctx._check(_lib.lib().omg_tc_gemm_bench(ctx.h, m, n, k, split, 200, C.byref(ms)), "omg_tc_gemm_bench")
        tf = 2.0 * m * n * k / (ms.value * 1e-3) / 1e12
        out[name] = {"us": 1e3 * ms.value, "tflops": tf, "frac_of_bf16_peak": tf / peak if peak else None}
    return out


def surrogate_leg(args, device, city=None):
    """The learned surrogate against the GPU tracer on the config-1 room family
    (shoebox, 6 x 3 absorptions, up to 4 apertures, poses): training data from
    the tracer (args.surrogate_train_rays per room), the tensor-core MLP
    ensemble trained on the GPU, then held-out rooms answered by both.
    Reported:
    - the training speed (TFLOP/s of the training steps, 3 x the forward
      FLOPs per sample) and the GEMMs alone at the training shapes;
    - the RT60 error of the surrogate's EDC against the tracer's (4096 rays),
      the Sabine formula's (the method without the network), and the noise
      floor of that judge: the tracer at 4096 rays against itself at another
      seed, and against 65,536 rays, on a subset of the test rooms;
    - the ensemble-spread gate swept: RT60 error of the ANSWERED rooms against
      the fraction answered, and the per-room time with the tracer's time for
      the rooms it falls back on;
    - ms per room of each, end to end through the C ABI with host buffers."""
    from omg_audio_gb300 import Context, TraceConfig
    from omg_audio_gb300 import surrogate as S
    ctx = Context(TraceConfig(device=device, n_bands=3, n_bins=2000, bin_dt=0.001, max_time=2.0, max_bounces=200,
                              energy_floor=1e-6, timeout_ms=120000))
    train_rays = args.surrogate_train_rays
    t0 = time.perf_counter()
    train = S.sample_rooms(args.surrogate_rooms, seed=1)
    bins, _ = S.trace_rooms(ctx, train, train_rays, seed=100)
    edc = S.edc_db(bins, 0.001)
    del bins
    t_data = time.perf_counter() - t0
    members = 4
    sur = S.RoomSurrogate(ctx, members=members)
    batch = 4096
    t0 = time.perf_counter()
    losses = sur.fit(train, edc, epochs=args.surrogate_epochs, batch=batch, lr=2e-3, lr_final=2e-5,
                     weight_decay=1e-4)
    t_train = time.perf_counter() - t0
    steps = (len(train) // batch) * args.surrogate_epochs
    train_tflops = 3.0 * FWD_FLOP * batch * steps * members / t_train / 1e12
    test = S.sample_rooms(args.surrogate_test, seed=99)
    S.trace_rooms(ctx, test.take(np.arange(64)), 4096, seed=7)      # warm-up
    sur.predict(test.take(np.arange(64)))
    t0 = time.perf_counter()
    bins_t, _ = S.trace_rooms(ctx, test, 4096, seed=7)
    t_trace = time.perf_counter() - t0
    t0 = time.perf_counter()
    pred, spread, ok = sur.predict(test)
    t_pred = time.perf_counter() - t0
    t0 = time.perf_counter()
    S.features(test)
    t_feat = time.perf_counter() - t0
    edc_t = S.edc_db(bins_t, 0.001)
    rt_t = S.rt60_from_edc(edc_t)
    rt_p = S.rt60_from_edc(pred)
    err = np.abs(rt_p / rt_t - 1.0)
    sab = np.abs(S.features(test)[:, S.SABINE_COLS] / rt_t - 1.0)
    n = len(test)
    # the judge's noise floor, on the first n_floor test rooms
    n_floor = min(n, args.surrogate_floor_rooms)
    sub = test.take(np.arange(n_floor))
    rt_b = S.rt60_from_edc(S.edc_db(S.trace_rooms(ctx, sub, 4096, seed=8)[0], 0.001))
    jr = args.surrogate_judge_rays
    rt_c = S.rt60_from_edc(S.edc_db(S.trace_rooms(ctx, sub, jr, seed=9)[0], 0.001))
    rt_d = S.rt60_from_edc(S.edc_db(S.trace_rooms(ctx, sub, jr, seed=10)[0], 0.001))
    nz_seed = np.abs(rt_b / rt_t[:n_floor] - 1.0)
    nz_65k = np.abs(rt_t[:n_floor] / rt_c - 1.0)
    nz_65k_65k = np.abs(rt_d / rt_c - 1.0)
    sur_65k = np.abs(rt_p[:n_floor] / rt_c - 1.0)

    def q(a, p):
        return float(np.nanpercentile(a, p))

    # the spread gate swept on the noise-floor rooms, judged by the tracer at
    # jr rays (the 4096-ray tracer's own p90 error is above 5 %): answered = in
    # the family and spread <= threshold; the rest fall back to the tracer
    inr = S.in_range(S.features(test))[:n_floor]
    spr = spread[:n_floor]
    tr_ms = 1e3 * t_trace / n
    su_ms = 1e3 * t_pred / n
    sweep = []
    for thr in [0.25, 0.5, 0.75, 1.0, 1.25, 1.5, 2.0, 3.0, 1e9]:
        ans = inr & (spr <= thr)
        fa = float(np.mean(ans))
        e_ans = sur_65k[ans] if ans.any() else np.full((1, 3), np.nan)
        per_room = su_ms + (1.0 - fa) * tr_ms
        sweep.append({"spread_db_max": thr if thr < 1e8 else None, "answered_frac": fa,
                      "rt60_err_median": q(e_ans, 50), "rt60_err_p90": q(e_ans, 90),
                      "ms_per_room_with_fallback": per_room, "speedup_with_fallback": tr_ms / per_room})
    ok5 = [r for r in sweep if r["rt60_err_p90"] <= 0.05]
    chosen = max(ok5, key=lambda r: r["answered_frac"]) if ok5 else None
    gemm = gemm_leg(ctx)
    city_leg = None
    if city is not None:
        # config 5's room/source pairs: every building x every source
        # the product's gate (RoomSurrogate.threshold_db), or the sweep's
        # stricter one: these rooms are not the test family's
        gate = sur.threshold_db
        if chosen and chosen["spread_db_max"] is not None:
            gate = min(gate, chosen["spread_db_max"])
        rooms = S.city_rooms(city.buildings, city.sources, city.absorption, city.window_frac)
        sur.predict(rooms.take(np.arange(64)))
        t0 = time.perf_counter()
        cedc, cspread, cok = sur.predict(rooms)
        t_cp = time.perf_counter() - t0
        ans = S.in_range(S.features(rooms)) & (cspread <= gate)
        fb = np.nonzero(~ans)[0]
        t0 = time.perf_counter()
        if len(fb):
            S.trace_rooms(ctx, rooms.take(fb), 4096, seed=31)
        t_fb = time.perf_counter() - t0
        t0 = time.perf_counter()
        cb, _ = S.trace_rooms(ctx, rooms, 4096, seed=31)
        t_all = time.perf_counter() - t0
        crt = S.rt60_from_edc(S.edc_db(cb, 0.001))
        crt_p = S.rt60_from_edc(cedc)
        cerr = np.abs(crt_p / crt - 1.0)[ans]
        # the answered pairs judged by the tracer at jr rays too, on a sample
        # (the 4096-ray tracer's own p90 error is about 10 %)
        aj = np.nonzero(ans)[0][:args.surrogate_floor_rooms // 2]
        cj, city_sweep = None, []
        if len(aj):
            rj = S.rt60_from_edc(S.edc_db(S.trace_rooms(ctx, rooms.take(aj), jr, seed=33)[0], 0.001))
            rj2 = S.rt60_from_edc(S.edc_db(S.trace_rooms(ctx, rooms.take(aj), jr, seed=34)[0], 0.001))
            ej = np.abs(crt_p[aj] / rj - 1.0)
            ejj = np.abs(rj2 / rj - 1.0)
            cj = {"pairs": int(len(aj)), "median": q(ej, 50), "p90": q(ej, 90),
                  "judge_vs_judge_other_seed": {"median": q(ejj, 50), "p90": q(ejj, 90)}}
            # the spread gate swept on the judged pairs, with the tracer's time
            # for the pairs each gate sends back
            tr_pair = t_all / len(rooms)
            for thr in [0.5, 0.75, 1.0, 1.25, 1.5, 2.0, 3.0]:
                a2 = cspread[aj] <= thr
                fa = float(np.mean(a2))
                e2 = ej[a2] if a2.any() else np.full((1, 3), np.nan)
                per = t_cp / len(rooms) + (1.0 - fa) * tr_pair
                city_sweep.append({"spread_db_max": thr, "answered_frac": fa, "rt60_err_median": q(e2, 50),
                                   "rt60_err_p90": q(e2, 90), "speedup_with_fallback": tr_pair / per})
        city_leg = {"pairs": len(rooms), "rooms": "per building x source: the ground-floor room (<= 15 x 11 x 3.5 m) "
                    "nearest the source, facade / ground / slab absorption at 250 Hz, 1 kHz, 4 kHz, perimeter walls "
                    "with their windows as apertures", "spread_gate_db": gate,
                    "answered_frac": float(np.mean(ans)), "fallback_pairs": int(len(fb)),
                    "surrogate_ms": 1e3 * t_cp, "fallback_tracer_ms": 1e3 * t_fb,
                    "ms_with_fallback": 1e3 * (t_cp + t_fb), "tracer_all_pairs_ms": 1e3 * t_all,
                    "speedup_with_fallback": t_all / (t_cp + t_fb),
                    "answered_rt60_err_vs_tracer_4096": {"median": q(cerr, 50), "p90": q(cerr, 90)},
                    "answered_rt60_err_vs_judge": cj, "spread_gate_sweep_vs_judge": city_sweep}
    ctx.close()
    return {
        "family": "shoebox 4-16 x 4-12 x 2.5-6 m, absorption in [0.02,0.4] x 6 surfaces x 3 bands (half the rooms "
                  "uniform and independent, half scattered around a log-uniform room level), scattering 0.1, "
                  "0-4 apertures 1.5 x 2 m with openness U[0,1], poses >= 1 m from walls",
        "network": "38 -> 256 x4 (GELU) -> 192 (64 log-time EDC points x 3 bands), 4-member ensemble, BF16 "
                   "tcgen05 GEMMs, FP32 accumulate and master weights, AdamW",
        "train_rooms": len(train), "train_rays": train_rays, "epochs": args.surrogate_epochs,
        "data_s": t_data, "train_s": t_train, "final_loss": float(np.mean(losses[:, -1])),
        "train_tflops": train_tflops,
        "train_flops_note": "3 x 510,976 FLOP per sample per member (forward, input and weight gradients)",
        "gemm": gemm,
        "test_rooms": n, "judge_rays": 4096,
        "rt60_err_median": float(np.nanmedian(err)), "rt60_err_p90": q(err, 90),
        "frac_rooms_all_bands_within_5pct": float(np.mean(np.nan_to_num(err, nan=1.0).max(1) <= 0.05)),
        "sabine_rt60_err_median": float(np.nanmedian(sab)),
        "edc_rmse_db": float(np.sqrt(np.mean((pred - edc_t) ** 2))),
        "judge_noise_floor": {
            "rooms": n_floor,
            "tracer_4096_vs_4096_other_seed": {"median": q(nz_seed, 50), "p90": q(nz_seed, 90)},
            "judge_rays": jr,
            "tracer_4096_vs_judge": {"median": q(nz_65k, 50), "p90": q(nz_65k, 90)},
            "judge_vs_judge_other_seed": {"median": q(nz_65k_65k, 50), "p90": q(nz_65k_65k, 90)},
            "surrogate_vs_judge": {"median": q(sur_65k, 50), "p90": q(sur_65k, 90)}},
        "spread_gate_sweep": sweep,
        "spread_gate_judge": f"the tracer at {jr} rays on the first {n_floor} test rooms",
        "chosen_gate": chosen,
        "p90_target_met": chosen is not None,
        "city_pairs": city_leg,
        "tracer_ms_per_room": tr_ms, "surrogate_ms_per_room": su_ms,
        "speedup": t_trace / t_pred, "surrogate_features_ms_per_room": 1e3 * t_feat / n,
        "timing": "wall clock of the calls with host buffers: trace_rooms (batched jobs, echograms down) vs "
                  "RoomSurrogate.predict (input features, omg_surrogate_query, decay curves down); with "
                  "fallback: the surrogate's time per room plus the tracer's for the share it falls back on",
    }


def early_leg(args, device, case):
    """World early reflections on the 40-room scene (its reference SAH tree):
    per listener, chain discovery (768 fan rays x 6 rotations) and the batched
    exact solve of every (source, chain) pair for the 64 sources, through the C
    ABI with host buffers; the oracle's single-thread solve of the same pairs
    beside it, and the number of pairs whose result differs."""
    from omg_audio_gb300 import Context, MeshBuilder, TraceConfig, _lib
    from omg_audio_gb300.early import WorldEarly
    from oracle import oracle as O
    ctx = Context(TraceConfig(device=device, timeout_ms=60000))
    mb = MeshBuilder()
    case.recorder.replay(mb)
    scene = ctx.upload_builder(mb, 3, _lib.BVH_SAH)
    early = WorldEarly(ctx, scene)
    oe = O.Early(oracle_mesh(case))
    sources = [(8 * i, src) for i, (src, _) in enumerate(case.pairs)]
    listeners = [lis for (_, lis) in case.pairs[:args.early_listeners]]
    extras = [(mn, mx, m.transmission) for (mn, mx, m) in case.panels]
    no = (_lib.NO_SURF,) * 3
    disc_ms, solve_ms, cpu_s, pairs, solved, mismatch, cpu_pairs = [], [], 0.0, 0, 0, 0, 0
    for li, lis in enumerate(listeners):
        early.discover(lis, 768, 0)                       # warm-up
        t0 = time.perf_counter()
        found = set()
        for rot in range(6):
            found.update(early.discover(lis, 768, rot))
        disc_ms.append(1e3 * (time.perf_counter() - t0) / 6)
        chains = [(no, 0)] + sorted(found)[:399]
        early.solve(sources, chains, lis, extras)         # warm-up
        t0 = time.perf_counter()
        rec = early.solve(sources, chains, lis, extras)
        solve_ms.append(1e3 * (time.perf_counter() - t0))
        pairs += rec.size
        solved += int(rec["valid"].sum())
        # the oracle on a sample of the sources, one thread
        k = 8
        t0 = time.perf_counter()
        _, valid = oe.solve(sources[:k], chains, lis, extras, threads=1)
        cpu_s += time.perf_counter() - t0
        cpu_pairs += valid.size
        mismatch += int(np.sum(valid != rec["valid"][:k].astype(bool)))
    early.close()
    scene.release()
    ctx.close()
    gpu_pairs_s = pairs / (1e-3 * float(np.sum(solve_ms)))
    return {
        "scene": "the 40-room scene (reference SAH tree), its panes as blockers",
        "listeners": len(listeners), "sources": len(sources), "fan_rays": 768, "rotations": 6,
        "chains_per_listener": round(pairs / len(sources) / len(listeners), 1),
        "pairs": pairs, "solved": solved, "discover_ms_per_call": float(np.mean(disc_ms)),
        "solve_ms_per_call": float(np.mean(solve_ms)), "solve_pairs_per_s": gpu_pairs_s,
        "cpu_pairs_per_s": cpu_pairs / cpu_s, "cpu_threads": 1,
        "cpu_sample": f"8 of {len(sources)} sources per listener (f32 oracle)",
        "mismatched_pairs_in_cpu_sample": mismatch,
        "timing": "wall clock of the calls with host buffers (chains and sources up, records down)",
    }


def run_workload(args):
    """The other configurations, one JSON line each (not the headline):
    rooms256 = 256 independent uneven rooms in one batch (lognormal triangle
    counts 12-20k, rays 512-65536, 3 or 8 bands, 0.5-4 s at 1 ms);
    city = the 1 M-triangle procedural city, 16 sources x 1 M rays x 8 bands,
    4 s at 1 ms, plus the 512-ray dome fan of 1024 street listeners."""
    import torch
    torch.cuda.set_device(0)
    from omg_audio_gb300 import build as B
    B.build()
    line = workload_summary(args, args.workload, args.steps, args.warmup, shape=args.shape or None,
                            autotune=args.autotune)
    if line is not None:
        print(json.dumps(line), flush=True)
    return 0


# the tree builders by name: sah3 is built on the GPU, sah3-host is the same tree built on the host
BVH_KINDS = {"sah": 0, "lbvh": 1, "sah3": 2, "sah3-host": 3}


def workload_summary(args, workload, steps, warmup, case=None, shape=None, autotune=True):
    """One secondary configuration measured (see run_workload): segments/s of
    the trace part (CUDA events, L2 flushed before each step), the roofline by
    the reference traversal's bytes per segment (the f32 oracle on a sample,
    first-found rule, reference tree), the oracle's own rate, clocks."""
    import torch
    from omg_audio_gb300 import Context, DomeProbe, Job, MeshBuilder, TraceConfig, _lib
    from omg_audio_gb300 import workloads as W
    bvh = BVH_KINDS[args.bvh]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    t0 = time.perf_counter()
    upload_s = 0.0     # scene uploads alone: tessellation, tree build, device arrays
    oracle_jobs = []   # (mesh recorder or box, src, lis, n_rays, seed, n_bands, n_bins, max_time) for the CPU leg
    if workload == "shoebox12":
        case = W.shoebox12(seed=1)
        ctx = Context(TraceConfig(timeout_ms=60000, tie_mode=1, **CFG))
        mb = MeshBuilder()
        case.recorder.replay(mb)
        sc = ctx.upload_builder(mb, 3, bvh)
        jobs = [Job(case.src, case.lis, N_RAYS, seed=11, scene=sc)]
        oracle_jobs = [(case.recorder, case.src, case.lis, N_RAYS, 11, 3, CFG["n_bins"], CFG["max_time"])]
        desc = "shoebox12: 10 x 7 x 4 m room as 12 triangles, 4096 rays x 3 bands, 2000 x 1 ms bins, 200 bounces"
        dome = None
        prims = sc.info()["prims"]
    elif workload == "rooms256":
        rooms = W.room_batch(seed=3, n_rooms=256)
        ctx = Context(TraceConfig(timeout_ms=120000, tie_mode=1, n_bins=4000, max_time=4.0, max_bounces=200,
                                  energy_floor=1e-6))
        scenes, jobs = [], []
        for k, r in enumerate(rooms):
            mb = MeshBuilder()
            r.recorder.replay(mb)
            tu = time.perf_counter()
            sc = ctx.upload_builder(mb, r.n_bands, bvh)
            upload_s += time.perf_counter() - tu
            scenes.append(sc)
            jobs.append(Job(r.src, r.lis, r.n_rays, seed=100 + k, scene=sc, n_bands=r.n_bands, n_bins=r.n_bins,
                            max_time=r.max_time))
            if k < 16:
                oracle_jobs.append((r.recorder, r.src, r.lis, r.n_rays, 100 + k, r.n_bands, r.n_bins, r.max_time))
        desc = ("rooms256: 256 rooms, triangles lognormal (median 2k, 12-20k), rays lognormal 512-65536 "
                f"({sum(j.n_rays for j in jobs)} in all), bands 3 or 8, 0.5-4 s at 1 ms, one batch")
        dome = None
        prims = sum(sc.info()["prims"] for sc in scenes)
    else:
        case = case or W.city(seed=5)
        ctx = Context(TraceConfig(timeout_ms=300000, tie_mode=1, n_bands=case.n_bands, n_bins=4000, bin_dt=0.001,
                                  max_time=4.0, max_bounces=200, energy_floor=1e-6))
        mb = MeshBuilder()
        case.recorder.replay(mb)
        tu = time.perf_counter()
        scene = ctx.upload_builder(mb, case.n_bands, bvh)
        upload_s = time.perf_counter() - tu
        prims = scene.info()["prims"]
        jobs = [Job(tuple(s_), tuple(l_), args.city_rays, seed=500 + k, scene=scene)
                for k, (s_, l_) in enumerate(zip(case.sources, case.listeners))]
        dome = DomeProbe(ctx, scene, (), n_fan=512)
        oracle_jobs = [(case.recorder, tuple(case.sources[0]), tuple(case.listeners[0]), 4096, 500, case.n_bands,
                        4000, 4.0)]
        desc = (f"city: {case.recorder.n_tris} triangles ({prims} primitives), 16 sources x {args.city_rays} rays "
                f"x 8 bands, 4 s at 1 ms, 200 bounces, floor 1e-6, + 512-ray dome fans of "
                f"{len(case.dome_eyes)} listeners")
    setup_s = time.perf_counter() - t0
    ctx.set_stream(stream.cuda_stream)
    batch = ctx.batch(jobs)
    if shape:
        batch.set_shape(**json.loads(shape))
        tune = batch.shape()
    else:
        tune = batch.autotune(reps=1) if autotune else batch.shape()
    for _ in range(max(warmup, 1)):
        batch.launch()
    torch.cuda.synchronize()
    if args.profile:
        # small case for a profiler: the launches only, nothing timed or printed
        for _ in range(steps):
            batch.launch()
            if dome is not None:
                dome.submit(case.dome_eyes, n_rays=512, stream=stream.cuda_stream, want=2)
                torch.cuda.synchronize()
                dome.collect()
        torch.cuda.synchronize()
        return None
    ms, dms = [], []
    with ClockSampler(0) as clk:
        for _ in range(steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            batch.launch(1)
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
            if dome is not None:
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                dome.submit(case.dome_eyes, n_rays=512, stream=stream.cuda_stream, want=2)
                b.record(stream)
                torch.cuda.synchronize()
                dres = dome.collect()
                dms.append(a.elapsed_time(b))
    batch.launch()
    res = batch.read()
    segs = batch.segments()
    line = {"metric": "ray-segments/s", "workload": workload, "desc": desc, "prims": prims,
            "bvh": args.bvh, "setup_s": setup_s, "upload_s": upload_s, "steps": steps, "trace_ms": float(np.mean(ms)),
            "segments": segs, "value": segs / (float(np.mean(ms)) * 1e-3), "unit": "ray-segments/s",
            "autotune": tune, "clocks": clk.summary(),
            "rt60_range": [float(np.nanmin([np.min(rv.rt60) for _, rv in res])),
                           float(np.nanmax([np.max(rv.rt60) for _, rv in res]))]}
    # CPU leg: the f32 oracle (the reference's algorithm over the reference's
    # SAH tree) on a sample, all host threads and one; its traversal counters
    # give the reference's bytes per segment on this configuration
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    tot = {k: 0 for k in ("segments", "receiver_hits") + O.TRAV_KEYS}
    sec = sec1 = seg1 = 0.0
    for rec, src, lis, n_rays, seed, nb, n_bins, tmax in oracle_jobs:
        ob = O.MeshBuilder()
        rec.replay(ob, lambda m: O.Material.make(m.absorption, m.scattering, m.transmission))
        mesh = ob.build("f32")
        # the reference's algorithm: first-found closest hits on its own tree
        P = O.params(tie_mode=0, n_bands=nb, n_bins=n_bins, bin_dt=0.001, max_time=tmax, max_bounces=200,
                     energy_floor=1e-6)
        t0 = time.perf_counter()
        _, _, st = O.trace_mesh(mesh, src, lis, n_rays, energy=[1.0] * nb, P=P, seed=seed, threads=threads)
        sec += time.perf_counter() - t0
        for k in tot:
            tot[k] += st[k]
        t0 = time.perf_counter()
        _, _, s1 = O.trace_mesh(mesh, src, lis, n_rays, energy=[1.0] * nb, P=P, seed=seed, threads=1,
                                ray_end=min(n_rays, 256))
        sec1 += time.perf_counter() - t0
        seg1 += s1["segments"]
    seg = tot["segments"]
    if seg:
        nbm = max(r[5] for r in oracle_jobs)
        bseg, parts = bytes_per_segment(tot, nbm)
        peak, peak_kind = peaks()
        line["cpu_baseline"] = {"value": seg / sec, "unit": "ray-segments/s", "cores": threads, "kind": "port",
                                "one_thread": seg1 / sec1,
                                "sample": f"{len(oracle_jobs)} job(s) of the workload (f32 oracle, first-found "
                                          f"rule, reference tree)"}
        line["roofline"] = {"bound": "hbm", "bytes_per_segment": bseg, "achieved": line["value"] * bseg / 1e9,
                            "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                            "frac": line["value"] * bseg / 1e9 / peak, **parts}
    if dome is not None:
        dseg = dres["segments"]["escape_events"] + dres["segments"]["through_calls"]
        line["dome"] = {"eyes": len(case.dome_eyes), "ms": float(np.mean(dms)), "segments": dseg,
                        "segments_per_s": dseg / (float(np.mean(dms)) * 1e-3),
                        "sky_escape_frac": float(np.mean(dres["escape"]))}
    ctx.close()
    torch.cuda.set_stream(torch.cuda.default_stream())
    return line


def compact_summary(line):
    keep = {k: line[k] for k in ("desc", "prims", "bvh", "setup_s", "upload_s", "steps", "trace_ms", "segments", "value",
                                 "unit", "autotune", "clocks", "cpu_baseline", "dome") if k in line}
    rf = line.get("roofline", {})
    keep["roofline"] = {k: rf[k] for k in ("bytes_per_segment", "achieved", "peak", "unit", "frac", "n_node",
                                           "n_prim", "h", "formula") if k in rf}
    return keep


def run_gemm_profile(args):
    """A small case for a profiler: the surrogate's GEMM at its training shapes
    (omg_tc_gemm_bench, a few launches each), nothing printed."""
    import ctypes as C

    import torch
    torch.cuda.set_device(0)
    from omg_audio_gb300 import build as B
    B.build()
    from omg_audio_gb300 import Context, TraceConfig, _lib
    with Context(TraceConfig(device=0)) as ctx:
        ms = C.c_float()
        for (m, n, k, split) in ((4096, 256, 256, 1), (256, 256, 4096, 8)):
            ctx._check(_lib.lib().omg_tc_gemm_bench(ctx.h, m, n, k, split, max(1, args.steps), C.byref(ms)),
                       "omg_tc_gemm_bench")
    return 0


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from omg_audio_gb300 import build as B
    B.build()
    from omg_audio_gb300 import Context, DomeProbe, Job, MeshBuilder, TraceConfig
    from omg_audio_gb300 import _lib

    case = build_case()
    cfg = dict(CFG)
    if args.max_bounces:
        cfg["max_bounces"] = args.max_bounces
    ctx = Context(TraceConfig(device=local, timeout_ms=60000, tie_mode=1, tri_test=1 if args.watertight else 0,
                              **cfg))
    # a dedicated stream: the library launches on it and the events are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    mb = MeshBuilder()
    case.recorder.replay(mb)
    bvh = BVH_KINDS[args.bvh]
    tu = time.perf_counter()
    scene = ctx.upload_builder(mb, 3, bvh)
    upload_s = time.perf_counter() - tu
    jobs = [Job(src, lis, N_RAYS, seed=1000 + p, scene=scene, panel_offset=0, n_panels=len(case.panels))
            for p, (src, lis) in enumerate(case.pairs[:args.pairs])]
    batch = ctx.batch(jobs, case.panels)
    if args.shape:
        batch.set_shape(**json.loads(args.shape))
        tune = batch.shape()
    else:
        tune = batch.autotune(reps=1) if args.autotune else None
    dome = DomeProbe(ctx, scene, case.glass, n_fan=DOME_RAYS)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step(ev=None):
        """One step on one stream: the batch (clear + trace, then finalize +
        reverb), then the 64 dome fans."""
        start = torch.cuda.Event(enable_timing=True) if ev is None else ev[0]
        start.record(stream)
        batch.launch(1)
        if ev:
            ev[1].record(stream)
        batch.launch(2)
        dome.submit(case.listeners, n_rays=DOME_RAYS, stream=stream.cuda_stream)
        if ev:
            ev[2].record(stream)

    for _ in range(max(args.warmup, 0)):
        step()
        torch.cuda.synchronize()
        dome.collect()
    torch.cuda.synchronize()
    if args.profile:
        # small case for a profiler: the launches only, nothing timed or printed
        for _ in range(args.steps):
            step()
            torch.cuda.synchronize()
            dome.collect()
        return 0
    if ws > 1:
        dist.barrier()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    dome_ms = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        for k in range(args.steps):
            flush.zero_()
            step(evs[k])
            torch.cuda.synchronize()
            dres = dome.collect()
        # the dome fans alone (device time on their stream), for the record
        for k in range(args.steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            dome.submit(case.listeners, n_rays=DOME_RAYS, stream=stream.cuda_stream)
            b.record(stream)
            torch.cuda.synchronize()
            dome.collect()
            dome_ms.append(a.elapsed_time(b))
        torch.cuda.synchronize()
    trace_ms = np.array([e[0].elapsed_time(e[1]) for e in evs])
    step_ms = np.array([e[0].elapsed_time(e[2]) for e in evs])
    segments = batch.segments()
    dome_seg = dres["segments"]["escape_events"] + dres["segments"]["through_calls"]
    t_step = float(np.mean(step_ms))

    # end to end through the C ABI with host buffers: the dome submitted (eyes
    # up, fans, bins down), the batch call on the same stream (jobs up, trace,
    # echograms and reverb down), then the dome collected. One untimed call
    # first (it sets up the one-shot batch record); the reported time is the
    # mean over the steps, with the median and the maximum beside it.
    dome.submit(case.listeners, n_rays=DOME_RAYS, stream=stream.cuda_stream)
    ctx.trace_batch(jobs, case.panels)
    dome.collect()
    e2e_ms = []
    for k in range(max(1, args.steps)):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dome.submit(case.listeners, n_rays=DOME_RAYS, stream=stream.cuda_stream)
        ctx.trace_batch(jobs, case.panels)
        dome.collect()
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    h2d, d2h = ctx.io_bytes()
    d2h += 64 * 9 * (3 + 3) * 4 + 2 * 4 + 16
    h2d += 64 * 12
    t_step, e2e_mean = max_over_ranks([t_step, float(np.mean(e2e_ms))], ws)
    value = aggregate_rate(ws, segments + dome_seg, t_step)
    e2e = aggregate_rate(ws, segments + dome_seg, e2e_mean)

    line = None
    if rank == 0:
        # CPU baseline (the reference's algorithm: first-found hits on its own
        # tree, plus the fans) and bytes per segment from its traversal counters
        threads = os.cpu_count() or 1
        cpu = cpu_sample(case, args.ref_pairs, threads)
        bseg, parts = bytes_per_segment(cpu)
        peak, peak_kind = peaks()
        t_trace = float(np.mean(trace_ms)) * 1e-3
        achieved = segments * bseg / t_trace / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": config_of(scene.info()["prims"]),
            "tri_test": ("watertight (Woop, Benthin, Wald 2013) on the exact vertices" if args.watertight
                         else "the reference's Moller-Trumbore with its epsilons"),
            "tie_rule": "near-tie rule (tie_mode 1: lowest surface id among hits within 1e-6 relative t) on the "
                        f"{args.bvh} tree",
            "detail": {"bvh": args.bvh, "upload_s": upload_s, "segments_per_step": segments,
                       "dome_segments_per_step": dome_seg, "trace_ms": float(np.mean(trace_ms)), "step_ms": float(np.mean(step_ms)),
                       "step_ms_max": float(np.max(step_ms)), "dome_alone_ms": float(np.mean(dome_ms)),
                       "dome": "the 64 fans after the trace, on its stream", "autotune": tune,
                       "parallelism": f"replicas x{ws}" if ws > 1 else "1 GPU"},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "ms_per_step": e2e_mean, "ms_median": float(np.median(e2e_ms)),
                    "ms_max": float(np.max(e2e_ms)), "statistic": "mean of the steps"},
            "gpu_launches": int(args.steps * (batch.kernel_count() + 3)),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic(), "peak_kind": peak_kind,
                         "bytes_per_segment": bseg, "segments_per_launch": segments,
                         "trace_ms": float(np.mean(trace_ms)), **parts,
                         "counters_from": f"the f32 oracle's reference traversal (first-found, reference SAH tree) "
                                          f"on {args.ref_pairs} of {N_PAIRS} pairs: {cpu['segments']} segments",
                         "kernel": "the trace part of a step (persistent trace kernels, CUDA events on their "
                                   "stream)"},
            "cpu_baseline": {"value": (cpu["segments"] + cpu["dome_segments"]) / cpu["seconds"], "unit": UNIT,
                             "cores": threads, "kind": "port",
                             "sample": f"{args.ref_pairs} of {N_PAIRS} pairs x {N_RAYS} rays and their dome fans "
                                       f"(f32 oracle, the reference's first-found rule and tree, {threads} threads)"},
            "clocks": clk.summary(),
        }
        city = None
        if args.extra_workloads:
            from omg_audio_gb300 import workloads as W
            city = W.city(seed=5)
        if args.surrogate:
            line["surrogate"] = surrogate_leg(args, local, city)
        if args.early_listeners > 0:
            line["early"] = early_leg(args, local, case)
        if args.extra_workloads:
            # the other two tracer configurations, measured here too (a few
            # steps each; the full lines come from --workload rooms256 / city)
            for name in ("rooms256", "city"):
                line[name] = compact_summary(workload_summary(args, name, args.extra_steps, 1,
                                                              case=city if name == "city" else None))
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--bvh", choices=list(BVH_KINDS), default=None,
                    help="sah: the reference's tree (host); sah3: three-axis binned SAH built on the GPU (default); "
                         "sah3-host: the same tree built on the host; lbvh: Morton LBVH built on the GPU")
    ap.add_argument("--ref-pairs", type=int, default=64)
    ap.add_argument("--pairs", type=int, default=N_PAIRS, help="pairs traced per step (default: the workload's 64)")
    ap.add_argument("--profile", action="store_true", help="launches only (a small case under a profiler)")
    ap.add_argument("--profile-gemm", action="store_true",
                    help="the surrogate's GEMM at two training shapes, --steps launches each (for a profiler)")
    ap.add_argument("--no-surrogate", dest="surrogate", action="store_false",
                    help="skip the surrogate leg (train on tracer data, compare with the tracer)")
    ap.add_argument("--early-listeners", type=int, default=8,
                    help="listeners of the world early-reflection leg (0 skips it)")
    ap.add_argument("--surrogate-rooms", type=int, default=131072, help="training rooms (1 M: the full config)")
    ap.add_argument("--surrogate-epochs", type=int, default=120)
    ap.add_argument("--surrogate-test", type=int, default=16384, help="held-out rooms")
    ap.add_argument("--surrogate-train-rays", type=int, default=8192,
                    help="tracer rays per training room (the labels' Monte-Carlo noise is the loss floor)")
    ap.add_argument("--surrogate-floor-rooms", type=int, default=1024,
                    help="test rooms traced again (another seed; --surrogate-judge-rays) for the judge's noise floor")
    ap.add_argument("--surrogate-judge-rays", type=int, default=131072,
                    help="rays of the low-noise judge the spread gate is swept against")
    ap.add_argument("--max-bounces", type=int, default=0,
                    help="profiling variant: cap the bounces (0: the workload's 200)")
    ap.add_argument("--shape", default="",
                    help="launch shape as JSON (omg_tune_result fields), instead of the autotuner")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="skip the launch-shape autotuner (it runs once, before the warm-up)")
    ap.add_argument("--workload", choices=["multiroom", "shoebox12", "rooms256", "city"], default="multiroom",
                    help="multiroom: the headline (default); rooms256 and city print their own line")
    ap.add_argument("--city-rays", type=int, default=1 << 20, help="rays per source of the city workload")
    ap.add_argument("--watertight", action="store_true",
                    help="the watertight ray-triangle test (omg_params.tri_test 1) instead of the reference's")
    ap.add_argument("--no-extra-workloads", dest="extra_workloads", action="store_false",
                    help="skip the rooms256 and city summaries of the headline line")
    ap.add_argument("--extra-steps", type=int, default=3, help="timed steps of each extra workload")
    args = ap.parse_args()
    if args.bvh is None:
        args.bvh = "sah3"
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_gemm:
        return run_gemm_profile(args)
    if args.workload != "multiroom":
        return run_workload(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
