"""Benchmark: ray-traced coverage (Rx-paths/s) on GB300.

Headline workload "coverage-128": a 12 x 8 x 3 m room with 20 seeded
floor-standing boxes (2172 triangles, reflection coefficients U[0.3, 0.7]),
a 16-element half-wavelength ULA at 60 GHz, a 128 x 128 Rx grid at 1.5 m,
a 1000 x 1000 forward launch and up to 2 reflections.  One step is one
channel build (Tx/Rx BVH builds + stage 1 + all stage-2 rounds) on a scene
whose triangle BVH is kept resident, as a user of the Scene API does.
Rx-paths = successful backward verifications (the reference's stats[0]).

Also reported (in "secondary"), each with its own roofline or baseline: the
plain phase-map objective (S=16, M=1024, R=4096, C=1) as objective+grad
evals/s; the 60-code codebook objective on tensor cores at 4,096 and 65,536
Rx; the ms-256 channel set (50k triangles, a 32x32 metasurface, 256x256 Rx,
3 reflections) with the objective on its traced channels; surrogate-screened
placement annealing against the plain traced loop (two-room study); 64
batched metasurface placements in a 200k-triangle building.  Every
objective figure carries its error against the FP64 oracle.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--only tracer|objective|codes|ms|surrogate|batch]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "coverage Rx-paths/s"
UNIT = "Rx-paths/s"
WORKLOAD = ("coverage-128: 12x8x3 m room + 20 boxes (2172 tris), 16-el ULA @60 GHz, "
            "128x128 Rx at 1.5 m, 1000x1000 launch, max_reflection=2")
# Ideal-BVH work of one closest-hit query (leaf-4 tree: 2 ceil(log2 ceil(N/4))
# slab tests of 18 flop + 4 primitive tests): 520 flop on the 2172-triangle
# scene (40-flop triangle tests); a stage-1 query also walks the 16,384 Rx
# spheres (24 slab tests + 4 20-flop sphere tests = 512 flop).
FLOP_PER_SEGMENT = 520
FLOP_PER_SEGMENT_FWD = 520 + 512
RECORD_BYTES = 60  # one forward record of the reference (Path + grid index)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi takes a moment to start: begin timing once it samples
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def profile_value(name, key):
    """A measured figure from a committed ncu summary under profiles/ (a line
    'key: N'), or None."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.strip().startswith(key + ":"):
                return int(line.split(":", 1)[1].strip())
    return None


def stage2_traffic():
    """DRAM bytes (read + write) of k_stage2 over one coverage-128 trace."""
    return profile_value("k_stage2_coverage128_traffic.md", "traffic_bytes_per_trace")


def stage1_traffic():
    """DRAM bytes (read + write) of one k_stage1 launch on coverage-128."""
    return profile_value("k_stage1_coverage128_traffic.md", "traffic_bytes_per_launch")


def kernel_launches(stats, aabbs_given):
    """Kernels of one trace call: 2 sphere BVH builds (7 each, plus the AABB
    kernel when the caller gives none), stage 1 + popcount, 4 per round,
    the finalize pass."""
    n = 14 + (0 if aabbs_given else 2) + 2 + 4 * stats["rounds"] + (1 if stats["fwd_records"] else 0)
    return n


def cpu_tracer_sample(cfg, threads):
    import oracle
    t0 = time.perf_counter()
    _, st, _ = oracle.trace_channel(cfg["tris"], cfg["mat"], cfg["mat_prop"], cfg["src"],
                                    cfg["dst"], cfg["params"], nthreads=threads)
    dt = time.perf_counter() - t0
    return st["rx_paths"], dt


def aggregate_over_ranks(torch, dist, device, elapsed, units):
    """Whole-job figures of N independent replicas (one seeded scene per
    rank, no collective on the data path): the slowest rank's elapsed time
    and the units all ranks processed.  dist is None for one process."""
    if dist is None:
        return elapsed, units
    t = torch.tensor([float(elapsed)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t), float(u)


def run_reference(args, rank, world):
    """The reference path's CPU restatement (oracle port, all host threads)."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from automs_gb300 import scenes
    cfg = scenes.coverage_config("coverage-128", seed=0)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_tracer_sample(cfg, threads)
    tot_p, tot_t = 0, 0.0
    for _ in range(args.steps):
        p, t = cpu_tracer_sample(cfg, threads)
        tot_p += p
        tot_t += t
    v = tot_p / tot_t
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic", "config": {"workload": WORKLOAD},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "one full coverage-128 build per step (C oracle, OpenMP)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def fp64_errors(Hd, Ha, Hr, phi, W, w, loss, gW, gphi):
    """Error of one objective evaluation (loss, dL/dW, dL/dphi from the GPU)
    against the FP64 oracle on the same channels: relative error of the loss
    and max-abs error of each gradient over the gradient's largest entry.
    Run after the timed region; the oracle is the checker here."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import objective_oracle as OO
    c = lambda t: t.detach().cpu().numpy()
    C = W.shape[0]
    lo, gWo, gpo = OO.objective_from_weights(c(Hd), c(Ha), c(Hr), c(phi), c(W), w,
                                             np.zeros(C, bool))
    g1, g2 = c(gW).reshape(gWo.shape), c(gphi)
    return {"loss": abs(float(loss) - lo) / abs(lo),
            "grad_W": float(np.abs(g1 - gWo).max() / np.abs(gWo).max()),
            "grad_phi": float(np.abs(g2 - gpo).max() / np.abs(gpo).max()),
            "vs": "FP64 oracle, same channels, one evaluation"}


def objective_bench(torch, steps, flush, cpu_baseline=False):
    """Plain objective fwd+bwd, S=16 M=1024 R=4096 C=1, through the C ABI.

    Eight independent channel sets (274 MB, more than L2) are evaluated in
    turn, so every evaluation streams its channels from HBM; the eight calls
    are captured once in a CUDA graph and replayed, which removes the host
    launch cost from the device timing.  The headline uses an evaluation plan
    per channel set (ams_objective_plan_*, made once: the channels fixed over
    an optimization, as in optimize_model); the direct call
    (ams_objective_fwd_bwd on the reference-orientation arrays) is timed
    beside it."""
    import ctypes as C

    from automs_gb300._lib import call, lib
    L = lib()
    rng = np.random.Generator(np.random.PCG64(1))
    S, M, R = 16, 1024, 4096
    NSET = 8
    lam = 3e8 / 60e9

    def cn(*sh):
        d = rng.uniform(2.0, 15.0, size=sh)
        g = (rng.normal(size=sh) + 1j * rng.normal(size=sh)) / np.sqrt(2)
        return torch.as_tensor((g * lam / (4 * np.pi * d)).astype(np.complex64), device="cuda")
    sets = [(cn(S, R), cn(S, M), cn(M, R)) for _ in range(NSET)]
    phi = torch.as_tensor(rng.uniform(0, 2 * np.pi, M).astype(np.float32), device="cuda")
    wv = rng.normal(size=S) + 1j * rng.normal(size=S)
    W = torch.as_tensor((wv / np.linalg.norm(wv)).astype(np.complex64)[None], device="cuda")
    loss = torch.empty(NSET, device="cuda")
    gW = torch.empty(NSET, 1, S, dtype=torch.complex64, device="cuda")
    gphi = torch.empty(NSET, M, device="cuda")
    P = lambda t: C.c_void_p(t.data_ptr())
    z = C.c_void_p(0)
    st = torch.cuda.Stream()
    plans = []
    t0 = time.perf_counter()
    for Hd, Ha, Hr in sets:
        h = C.c_void_p()
        call("ams_objective_plan_create", P(Hd), P(Ha), P(Hr), S, M, R, 1,
             C.c_void_p(st.cuda_stream), C.byref(h))
        plans.append(h)
    st.synchronize()
    t_plan = (time.perf_counter() - t0) / NSET

    def ev_plan():
        for i, h in enumerate(plans):
            call("ams_objective_plan_fwd_bwd", h, P(phi), float(2 * np.pi), P(W), 1, 1.0 / R, z,
                 P(loss[i]), P(gW[i]), P(gphi[i]), z, z, C.c_void_p(st.cuda_stream))

    def ev_direct():
        for i, (Hd, Ha, Hr) in enumerate(sets):
            call("ams_objective_fwd_bwd", P(Hd), P(Ha), P(Hr), P(phi), float(2 * np.pi), P(W), S,
                 M, R, 1, 1.0 / R, z, P(loss[i]), P(gW[i]), P(gphi[i]), z, z,
                 C.c_void_p(st.cuda_stream))

    def timed(fn, reps):
        with torch.cuda.stream(st):
            for _ in range(3):
                fn()
            st.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=st):
                fn()
            for _ in range(3):
                g.replay()
            st.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            flush()
            e0.record(st)
            for _ in range(reps):
                g.replay()
            e1.record(st)
            st.synchronize()
        return e0.elapsed_time(e1) / (reps * NSET)
    reps = max(1, steps // NSET)
    t = timed(ev_plan, reps)
    loss_plan = loss.clone()
    st.synchronize()
    err = fp64_errors(*sets[0], phi, W, 1.0 / R, loss[0], gW[0], gphi[0])
    t_direct = timed(ev_direct, reps)
    rel = float(((loss_plan - loss).abs() / loss.abs()).max())
    for h in plans:
        L.ams_objective_plan_destroy(h)
    cpu = None
    if cpu_baseline:
        # the reference's method (PyTorch complex64 + autograd, go.py:107-245)
        # on the host cores, same shapes, 20 evaluations
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import objective_oracle as OO
        threads = os.cpu_count() or 1
        torch.set_num_threads(threads)
        Hd, Ha, Hr = (x.cpu() for x in sets[0])
        phc, Wc = phi.cpu(), W.cpu()
        for _ in range(3):
            OO.torch_objective_step(torch, Hd, Ha, Hr, phc, Wc, 1.0 / R)
        n_cpu = 20
        t0 = time.perf_counter()
        for _ in range(n_cpu):
            OO.torch_objective_step(torch, Hd, Ha, Hr, phc, Wc, 1.0 / R)
        cpu = {"value": n_cpu / (time.perf_counter() - t0), "unit": "evals/s", "cores": threads,
               "kind": "port",
               "sample": "20 evaluations of the reference's method restated "
                         "(PyTorch complex64 + autograd, checked against the FP64 oracle, "
                         "which is pinned to the reference Model's outputs) on the host CPU, "
                         "same S/M/R"}
    bytes_alg = 8 * (R * M + M * S + R * S)
    hbm, kind = peaks()
    achieved = bytes_alg / (t * 1e-3) / 1e9
    return {"metric": "objective+grad evals/s", "value": 1e3 / t, "unit": "evals/s",
            "ms_per_eval": t, "evals": reps * NSET,
            "config": {"S": S, "M": M, "R": R, "C": 1,
                       "l2": "8 channel sets (274 MB) evaluated in turn, CUDA-graph replay",
                       "path": "evaluation plan per channel set (transposed FP32 copy)",
                       "plan_create_ms": t_plan * 1e3},
            "direct_call": {"value": 1e3 / t_direct, "ms_per_eval": t_direct,
                            "max_rel_loss_diff": rel},
            "rel_err_vs_fp64": err,
            "cpu_baseline": cpu,
            "roofline": {"bound": "hbm", "kernel": "k_obj_stream_t", "achieved": achieved,
                         "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": profile_value("k_obj_stream_c1_traffic.md",
                                                  "traffic_bytes_per_launch"),
                         "algorithmic_bytes": bytes_alg, "peak_kind": kind,
                         "note": "achieved = algorithmic bytes / whole-evaluation time"},
            "gpu_launches_per_eval": 3}


def objective_codes_bench(torch, R=4096, C=60, nset=4, reps=20):
    """Codebook objective+grad (C codes, the reference Model's use) on the
    tensor-core plan path (two tcgen05 3xBF16 GEMMs per evaluation) and on the
    FP32 CUDA-core path, S=16, M=1024.  `nset` channel sets are evaluated in
    turn so that the plan operands (about 8 (M+S) R bytes each way) exceed L2;
    each evaluation is replayed from a CUDA graph."""
    import ctypes as C_

    from automs_gb300._lib import call, lib
    L = lib()
    rng = np.random.Generator(np.random.PCG64(2))
    S, M = 16, 1024
    lam = 3e8 / 60e9

    def cn(*sh):
        d = rng.uniform(2.0, 15.0, size=sh)
        g = (rng.normal(size=sh) + 1j * rng.normal(size=sh)) / np.sqrt(2)
        return torch.as_tensor((g * lam / (4 * np.pi * d)).astype(np.complex64), device="cuda")
    P = lambda t: C_.c_void_p(t.data_ptr())
    st = torch.cuda.Stream()
    sets, plans = [], []
    for _ in range(nset):
        Hd, Ha, Hr = cn(S, R), cn(S, M), cn(M, R)
        h = C_.c_void_p()
        call("ams_objective_plan_create", P(Hd), P(Ha), P(Hr), S, M, R, C, C_.c_void_p(st.cuda_stream),
             C_.byref(h))
        sets.append((Hd, Ha, Hr))
        plans.append(h)
    phi = torch.as_tensor(rng.uniform(0, 2 * np.pi, M).astype(np.float32), device="cuda")
    th = rng.uniform(0, 2 * np.pi, size=(C, S))
    W = torch.as_tensor(np.exp(-1j * th).astype(np.complex64), device="cuda")
    loss = torch.empty(nset, device="cuda")
    gW = torch.empty(nset, C, S, dtype=torch.complex64, device="cuda")
    gphi = torch.empty(nset, M, device="cuda")
    z = C_.c_void_p(0)

    def ev_tc():
        for i, h in enumerate(plans):
            call("ams_objective_plan_fwd_bwd", h, P(phi), float(2 * np.pi), P(W), C, 1.0 / R, z,
                 P(loss[i]), P(gW[i]), P(gphi[i]), z, z, C_.c_void_p(st.cuda_stream))

    def ev_cc():
        for i, (Hd, Ha, Hr) in enumerate(sets):
            call("ams_objective_fwd_bwd", P(Hd), P(Ha), P(Hr), P(phi), float(2 * np.pi), P(W), S,
                 M, R, C, 1.0 / R, z, P(loss[i]), P(gW[i]), P(gphi[i]), z, z,
                 C_.c_void_p(st.cuda_stream))

    def timed(fn, n):
        with torch.cuda.stream(st):
            for _ in range(3):
                fn()
            st.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=st):
                fn()
            for _ in range(3):
                g.replay()
            st.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for _ in range(n):
                g.replay()
            e1.record(st)
            st.synchronize()
        return e0.elapsed_time(e1) / (n * nset)
    t_tc = timed(ev_tc, reps)
    loss_tc = loss.clone()
    st.synchronize()
    err = fp64_errors(*sets[0], phi, W, 1.0 / R, loss[0], gW[0], gphi[0])
    t_cc = timed(ev_cc, max(2, reps // 4))
    rel = float(((loss_tc - loss).abs() / loss.abs()).max())
    K = M + S
    Kp = -(-2 * K // 64) * 64
    Rp = -(-R // 128) * 128
    Np = -(-K // 128) * 128
    K2p = -(-2 * R // 64) * 64
    op_bytes = 4 * (Rp * Kp + Np * K2p)                 # B_y and B_g, hi + lo
    mma_flop = 3 * 2 * 128 * (Kp * Rp + K2p * Np)        # executed on the tensor pipe
    alg_flop = 16 * C * K * R                            # complex fwd + adjoint
    hbm, kind = peaks()
    bf16 = 1913.2
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            bf16 = float(json.load(f)["bf16_tflops"])
    except Exception:
        pass
    for h in plans:
        L.ams_objective_plan_destroy(h)
    gbs = op_bytes / (t_tc * 1e-3) / 1e9
    tfl = mma_flop / (t_tc * 1e-3) / 1e12
    return {"metric": f"objective+grad evals/s, {C}-code codebook", "value": 1e3 / t_tc,
            "unit": "evals/s", "ms_per_eval": t_tc,
            "config": {"S": S, "M": M, "R": R, "C": C,
                       "l2": f"{nset} channel sets in turn ({nset * op_bytes / 1e6:.0f} MB of "
                             "plan operands), CUDA-graph replay"},
            "cuda_core_path": {"value": 1e3 / t_cc, "ms_per_eval": t_cc},
            "speedup_vs_cuda_core": t_cc / t_tc,
            "rel_err_vs_fp64": err,
            "max_rel_loss_diff_vs_cuda_core": rel,
            "algorithmic_tflops": alg_flop / (t_tc * 1e-3) / 1e12,
            "roofline": {"bound": "hbm", "kernel": "k_cgemm3 (both GEMMs)", "achieved": gbs,
                         "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                         "bytes_per_eval": op_bytes, "peak_kind": kind,
                         "traffic": profile_value("k_cgemm3_codebook60_r65536.md",
                                                  "traffic_bytes_per_eval")
                         if R == 65536 else None,
                         "note": "achieved = plan operand bytes / whole-evaluation time"},
            "roofline_tensor": {"bound": "tensor", "achieved": tfl, "peak": bf16,
                                "unit": "TFLOP/s", "frac": tfl / bf16,
                                "mma_flop_per_eval": mma_flop, "peak_kind": "measured bf16 burst"}}


def surrogate_bench(torch, n_train=1500, n_val=200, n_cand=5000, top_frac=0.05, n_scenes=16,
                    test_scenes=(3, 11)):
    """Surrogate-screened placement search against the plain tracer-judged
    annealing loop (placement.TwoRoomStudy: 16 seeded two-room floors, AP in
    room A before the door, 64x64 Rx over room B, one reflection so that
    most of room B is dark without a metasurface, metasurfaces of 32x32 to
    64x64 on room A's other walls relaying through the door; a sample = the
    three traces + 12 Adam steps of the phase map; target = the 64x64 gain
    map in dB).  The MLP
    72 -> 4x512 -> 4096 (BF16 tcgen05 GEMMs, FP32 master weights) trains on
    n_train traced samples and is scored on n_val others against the
    constant-mean predictor.  Then per test scene, from one random start: a
    surrogate-scored annealing chain over n_cand candidates whose top
    top_frac the tracer judges, against the plain annealing loop with every
    move traced, given the same number of traces."""
    from automs_gb300 import placement, surrogate
    study = placement.TwoRoomStudy(n_scenes=n_scenes, seed=3, rx=(64, 64), launch=250,
                                   max_reflection=1, sizes=(32, 64))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    Xtr, Ytr, _ = study.dataset(n_train, seed=1, workers=4)
    torch.cuda.synchronize()
    t_sample = (time.perf_counter() - t0) / n_train
    Xva, Yva, _ = study.dataset(n_val, seed=2, workers=4)
    mu, sd = Ytr.mean(0), Ytr.std() + 1e-6
    net = surrogate.MLP([Xtr.shape[1], 512, 512, 512, 512, Ytr.shape[1]], max_batch=4096, seed=0)
    # about the same number of optimiser steps and the same final learning
    # rate whatever the training-set size (400 epochs at 1,500 samples)
    epochs = max(60, round(400 * 1500 / n_train))
    t0 = time.perf_counter()
    hist = net.fit(torch.as_tensor(Xtr).cuda(), torch.as_tensor((Ytr - mu) / sd).cuda(),
                   epochs=epochs, batch=64, lr=1e-3, lr_decay=0.995 ** (400 / epochs))
    torch.cuda.synchronize()
    t_fit = time.perf_counter() - t0
    mu_t = torch.as_tensor(mu, device="cuda")

    def predict(X):
        return net(X) * sd + mu_t
    pva = predict(torch.as_tensor(Xva).cuda()).cpu().numpy()
    err_net = float(np.median(np.abs(pva - Yva)))
    err_mean = float(np.median(np.abs(mu[None] - Yva)))
    lit = np.abs(Yva) >= 1.0  # cells the metasurface moves by a dB or more
    err_lit = float(np.median(np.abs(pva - Yva)[lit])) if lit.any() else None
    err_lit_mean = float(np.median(np.abs(mu[None] - Yva)[lit])) if lit.any() else None
    by_gain = {}
    for thr in (3.0, 10.0):  # cells the metasurface lights by several dB
        m = Yva >= thr
        if m.any():
            by_gain[f"ge_{int(thr)}db"] = {
                "cells": float(m.mean()), "median_gain_db": float(np.median(Yva[m])),
                "net_median_abs_err_db": float(np.median(np.abs(pva - Yva)[m])),
                "mean_predictor_median_abs_err_db": float(np.median(np.abs(mu[None] - Yva)[m]))}
    s_true, s_pred = Yva.mean(1), pva.mean(1)
    err_score = float(np.median(np.abs(s_pred - s_true)))
    err_score_mean = float(np.median(np.abs(mu.mean() - s_true)))
    rank_corr = float(np.corrcoef(np.argsort(np.argsort(s_pred)),
                                  np.argsort(np.argsort(s_true)))[0, 1])
    rows = []
    for k in test_scenes:
        rng = np.random.Generator(np.random.PCG64(100 + k))
        start = study.random_params(rng, scene=k)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cands = placement.anneal_candidates(study, n_cand, rng, surrogate=predict, start=start)
        X = torch.as_tensor(np.stack([study.descriptor(q) for q in cands]), device="cuda")
        ps = placement.score(predict(X)).cpu().numpy()
        torch.cuda.synchronize()
        t_rank = time.perf_counter() - t0
        judged = np.argsort(-ps)[:max(1, int(round(top_frac * n_cand)))]
        # the judged placements are known once ranked: traced together
        t0 = time.perf_counter()
        gains = study.evaluate_many([cands[i] for i in judged], workers=4)
        best_s = max(float(placement.score(g)) for g in gains)
        torch.cuda.synchronize()
        t_judge = time.perf_counter() - t0
        _, plain_s, t_plain = placement.anneal_traced(study, len(judged),
                                                      np.random.Generator(np.random.PCG64(200 + k)),
                                                      start)
        rows.append(dict(scene=k, screened_best_db=best_s, plain_best_db=float(plain_s.max()),
                         screened_configs_per_s=n_cand / (t_rank + t_judge),
                         plain_configs_per_s=len(judged) / t_plain, judged=len(judged),
                         t_rank_s=t_rank, t_judge_s=t_judge, t_plain_s=t_plain))
    net.close()
    study.close()
    scr = float(np.mean([r["screened_configs_per_s"] for r in rows]))
    pln = float(np.mean([r["plain_configs_per_s"] for r in rows]))
    return {"metric": "placement configs/s, surrogate-screened annealing vs plain",
            "value": scr, "unit": "configs/s", "plain_configs_per_s": pln, "ratio": scr / pln,
            "surrogate_median_abs_err_db": err_net,
            "mean_predictor_median_abs_err_db": err_mean,
            "err_ratio_vs_mean_predictor": err_net / err_mean,
            "median_abs_gain_db": float(np.median(np.abs(Yva))),
            "cells_gain_ge_1db": float(lit.mean()),
            "placements_score_ge_0p5db": float((s_true >= 0.5).mean()),
            "median_abs_err_db_cells_ge_1db": [err_lit, err_lit_mean],
            "lit_cells": by_gain,
            "score_median_abs_err_db": [err_score, err_score_mean],
            "score_rank_correlation": rank_corr,
            "best_gain_db_screened_vs_plain": [[r["screened_best_db"], r["plain_best_db"]]
                                               for r in rows],
            "config": {"workload": "two-room NLOS study: 16 floors, 64x64 Rx in room B, "
                                   "1 reflection (57% of room B dark without a metasurface), "
                                   "MS 32x32-64x64 on room A walls, MLP 72-4x512-4096",
                       "train_samples": n_train, "val_samples": n_val, "candidates": n_cand,
                       "judged_per_scene": rows[0]["judged"],
                       "t_sample_s": t_sample,
                       "judge": "the ranked top 5% traced on 4 host threads / CUDA streams "
                                "(study.evaluate_many); the plain loop traces one move after "
                                "another",
                       "t_rank_judge_plain_s": [[r["t_rank_s"], r["t_judge_s"], r["t_plain_s"]]
                                                for r in rows],
                       "epochs": epochs, "t_fit_s": t_fit,
                       "fit_loss_first_last": [hist[0], hist[-1]]}}


def batch_bench(torch, n_place=64, workers=4, opt_steps=20):
    """Batched hyper-configs: n_place metasurface placements (16x16 to 64x64
    elements) on the outer walls of a seeded ~200k-triangle multi-room
    building, 256x256 Rx grid, 1000x1000 launches, 2 reflections; per
    placement the AP->Rx (metasurface as blackhole), AP->MS and MS->Rx traces
    and opt_steps objective+adjoint Adam steps on an evaluation plan.
    Placements run on `workers` host threads with one CUDA stream each."""
    from automs_gb300 import placement, scenes
    cfg = scenes.batch_config(n_place=n_place)
    # warm-up: one small placement (library load, first launches)
    small = min(range(n_place), key=lambda i: cfg["placements"][i]["size"])
    placement.batch_evaluate(cfg, [small], workers=1, opt_steps=2)
    res, wall = placement.batch_evaluate(cfg, list(range(n_place)), workers=workers,
                                         opt_steps=opt_steps)
    paths = sum(r["rx_paths"] for r in res)
    improved = sum(1 for r in res if r["loss_last"] < r["loss_first"])
    gain = [r["loss_first"] - r["loss_last"] for r in res]
    return {"metric": "batched hyper-configs/s (trace + objective+adjoint)", "value": n_place / wall,
            "unit": "configs/s", "wall_s": wall, "rx_paths_per_s": paths / wall,
            "config": {"workload": "multi-room building, 199,976 triangles, 16-element AP, "
                                   "256x256 Rx, 1000x1000 launch, 2 reflections",
                       "placements": n_place, "sizes": "16x16 to 64x64 (step 8)",
                       "workers": workers, "adam_steps": opt_steps},
            "mean_trace_s": float(np.mean([r["t_trace"] for r in res])),
            "mean_opt_s": float(np.mean([r["t_opt"] for r in res])),
            "placements_with_lower_loss": improved,
            "median_loss_decrease": float(np.median(gain)),
            "median_ms_share": float(np.median([r["ms_share"] for r in res]))}


def channel_ms_bench(torch, warmup, steps, flush):
    """Channel set with one 32x32 metasurface on a 50k-triangle scene, 256x256
    Rx grid, 3 reflections, 1000x1000 launches: the AP->Rx, AP->MS and MS->Rx
    traces on resident scenes (Rx-paths/s over the three), then objective+grad
    evaluations on the traced channels (S=16, M=1024, R=65536; H_r is 537 MB,
    more than L2, so every evaluation streams it from HBM)."""
    import ctypes as C

    from automs_gb300 import scenes, tracer
    from automs_gb300._lib import call
    cfg = scenes.channel_ms_config("ms-256")
    base = tracer.Scene(cfg["tris"], cfg["mat"], cfg["mat_prop"])
    bh = tracer.Scene(*scenes.with_blackholes(cfg["tris"], cfg["mat"], cfg["mat_prop"],
                                              [cfg["blackhole"]]))
    jobs = []
    for key, t in cfg["traces"].items():
        sc = bh if t["blackhole"] else base
        src = torch.as_tensor(t["src"], device="cuda")
        dst = torch.as_tensor(t["dst"], device="cuda")
        res = torch.zeros(src.shape[0] * src.shape[1], dst.shape[0] * dst.shape[1], 2,
                          device="cuda")
        jobs.append((key, sc, src, dst, tracer.params_from_dict(t["params"]), res))
    stream = torch.cuda.current_stream()
    per = {k: [] for k, *_ in jobs}
    for it in range(warmup + steps):
        for key, sc, src, dst, prm, res in jobs:
            flush()
            res.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _, st = sc.trace(src, dst, prm, result=res)
            e1.record(stream)
            torch.cuda.synchronize()
            if it >= warmup:
                per[key].append((e0.elapsed_time(e1), st))
    base.close()
    bh.close()
    traces = {}
    tot_ms, tot_paths = 0.0, 0
    for key, v in per.items():
        ms = sum(a for a, _ in v) / len(v)
        st = v[0][1]
        traces[key] = {"ms": round(ms, 2), "rx_paths": st["rx_paths"],
                       "ms_stage2": round(st["ms_stage2"], 2),
                       "acc_adds_per_verified_ray": (round(st["acc_adds"] / st["rx_paths"], 3)
                                                     if st["rx_paths"] else None)}
        tot_ms += ms
        tot_paths += st["rx_paths"]
    # objective + adjoint on the traced channels, reference orientation
    Hd, Ha, Hr = (r for _, _, _, _, _, r in jobs)
    S, M, R = Ha.shape[0], Ha.shape[1], Hd.shape[1]
    rng = np.random.Generator(np.random.PCG64(3))
    phi = torch.as_tensor(rng.uniform(0, 2 * np.pi, M).astype(np.float32), device="cuda")
    wv = rng.normal(size=S) + 1j * rng.normal(size=S)
    W = torch.as_tensor((wv / np.linalg.norm(wv)).astype(np.complex64)[None], device="cuda")
    loss = torch.empty(1, device="cuda")
    gW = torch.empty(1, S, dtype=torch.complex64, device="cuda")
    gphi = torch.empty(M, device="cuda")
    P = lambda t: C.c_void_p(t.data_ptr())

    def ev():
        call("ams_objective_fwd_bwd", P(Hd), P(Ha), P(Hr), P(phi), float(2 * np.pi), P(W), S,
             M, R, 1, 1.0 / R, C.c_void_p(0), P(loss), P(gW), P(gphi), C.c_void_p(0),
             C.c_void_p(0), C.c_void_p(stream.cuda_stream))
    for _ in range(5):
        ev()
    n_ev = 50
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(n_ev):
        ev()
    e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / n_ev
    torch.cuda.synchronize()
    err = fp64_errors(*(torch.view_as_complex(x) for x in (Hd, Ha, Hr)), phi, W, 1.0 / R,
                      loss[0], gW, gphi)
    bytes_alg = 8 * (R * M + M * S + R * S)
    hbm, kind = peaks()
    achieved = bytes_alg / (t * 1e-3) / 1e9
    return {"metric": "channel-set Rx-paths/s", "value": tot_paths / (tot_ms * 1e-3),
            "unit": "Rx-paths/s", "ms_per_set": tot_ms, "steps": steps,
            "config": {"workload": "ms-256: 50,028 triangles, 16-element ULA, 32x32 "
                       "metasurface, 256x256 Rx, 1000x1000 launch, 3 reflections",
                       "l2": "flushed before every trace (256 MB write)"},
            "traces": traces,
            "objective": {"metric": "objective+grad evals/s", "value": 1e3 / t,
                          "ms_per_eval": t, "S": S, "M": M, "R": R, "C": 1,
                          "l2": "H_r 537 MB > L2, back-to-back evaluations",
                          "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm,
                                       "unit": "GB/s", "frac": achieved / hbm,
                                       "algorithmic_bytes": bytes_alg, "peak_kind": kind},
                          "loss": float(loss), "rel_err_vs_fp64": err}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the codebook, channel-set and surrogate legs")
    ap.add_argument("--only", default="all",
                    choices=["all", "tracer", "objective", "ms", "codes", "surrogate", "batch"],
                    help="profiling aid: run only the named timed loop")
    ap.add_argument("--batch-n", type=int, default=64, help="placements of the batch leg")
    ap.add_argument("--batch-workers", type=int, default=4)
    ap.add_argument("--surrogate-train", type=int, default=1500,
                    help="traced training samples of the surrogate leg")
    ap.add_argument("--codes-r", type=int, default=0, choices=[0, 4096, 65536],
                    help="profiling aid: run the codebook leg at one Rx count only")
    ap.add_argument("--launch", type=int, default=0,
                    help="profiling aid: override the forward launch edge (default 1000)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from automs_gb300 import scenes, tracer

    cfg = scenes.coverage_config("coverage-128", seed=rank)
    if args.launch:
        cfg["params"]["launch_x"] = cfg["params"]["launch_y"] = args.launch
    if args.only == "ms":
        flushbuf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        print(json.dumps(channel_ms_bench(torch, 1, max(1, args.steps),
                                          lambda: flushbuf.fill_(1.0))))
        return
    if args.only == "batch":
        print(json.dumps(batch_bench(torch, n_place=args.batch_n, workers=args.batch_workers)))
        return
    if args.only == "surrogate":
        print(json.dumps(surrogate_bench(torch, n_train=args.surrogate_train)))
        return
    if args.only == "codes":
        if args.codes_r in (0, 4096):
            print(json.dumps(objective_codes_bench(torch, R=4096)))
        if args.codes_r in (0, 65536):
            print(json.dumps(objective_codes_bench(torch, R=65536, nset=1)))
        return
    if args.only == "objective":
        flushbuf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        print(json.dumps(objective_bench(torch, args.steps, lambda: flushbuf.fill_(1.0))))
        return
    scene = tracer.Scene(cfg["tris"], cfg["mat"], cfg["mat_prop"])
    src = torch.as_tensor(cfg["src"], device="cuda")
    dst = torch.as_tensor(cfg["dst"], device="cuda")
    params = tracer.params_from_dict(cfg["params"])
    S = src.shape[0] * src.shape[1]
    Rn = dst.shape[0] * dst.shape[1]
    result = torch.zeros(S, Rn, 2, device="cuda")
    flushbuf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def flush():
        flushbuf.fill_(1.0)

    for _ in range(args.warmup):
        result.zero_()
        scene.trace(src, dst, params, result=result)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    steps = []
    with ClockSampler(local) as clk:
        barrier()
        t_wall = time.perf_counter()
        for _ in range(args.steps):
            flush()
            result.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _, st = scene.trace(src, dst, params, result=result)
            e1.record(stream)
            steps.append((e0, e1, st))
        barrier()
        t_wall = time.perf_counter() - t_wall
    ms = [a.elapsed_time(b) for a, b, _ in steps]
    total_ms = sum(ms)
    paths = sum(s["rx_paths"] for _, _, s in steps)
    st0 = steps[0][2]
    total_ms, paths = aggregate_over_ranks(torch, dist if world > 1 else None, "cuda",
                                           total_ms, paths)
    value = paths / (total_ms * 1e-3)
    if args.only == "tracer":
        print(json.dumps({"metric": METRIC, "value": value, "ms_per_step": total_ms / args.steps,
                          "stats": {k: v for k, v in steps[0][2].items()}}))
        return

    # ---- end to end through the public API from host buffers
    h_tris = torch.as_tensor(cfg["tris"]).pin_memory()
    h_mat = torch.as_tensor(cfg["mat"]).pin_memory()
    h_mp = torch.as_tensor(cfg["mat_prop"]).pin_memory()
    h_src = torch.as_tensor(cfg["src"]).pin_memory()
    h_dst = torch.as_tensor(cfg["dst"]).pin_memory()
    h_out = torch.empty(S, Rn, 2, dtype=torch.float32).pin_memory()
    h2d = sum(t.numel() * t.element_size() for t in (h_tris, h_mat, h_mp, h_src, h_dst))
    d2h = h_out.numel() * 4
    e2e_paths, e2e_t = 0, 0.0
    for k in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sc = tracer.Scene(h_tris.cuda(non_blocking=True), h_mat.cuda(non_blocking=True),
                          h_mp.cuda(non_blocking=True))
        res, st = sc.trace(h_src.cuda(non_blocking=True), h_dst.cuda(non_blocking=True), params)
        h_out.copy_(res, non_blocking=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        sc.close()
        if k >= args.warmup:
            e2e_paths += st["rx_paths"]
            e2e_t += dt
    e2e_t, e2e_paths = aggregate_over_ranks(torch, dist if world > 1 else None, "cuda", e2e_t,
                                            e2e_paths)
    e2e = {"value": e2e_paths / e2e_t, "unit": UNIT, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h,
           "note": "Scene creation (copies + triangle BVH) + trace + result download per step"}

    obj = objective_bench(torch, 200, flush, cpu_baseline=not args.no_cpu_baseline and world == 1)
    secondary = [obj]
    if not args.no_secondary:
        secondary.append(objective_codes_bench(torch, R=4096))
        secondary.append(objective_codes_bench(torch, R=65536, nset=1))
        secondary.append(channel_ms_bench(torch, 1, 1, flush))
        secondary.append(surrogate_bench(torch, n_train=args.surrogate_train))
        secondary.append(batch_bench(torch))

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    clocks = clk.summary()
    hbm, peak_kind = peaks()
    k2_ms = st0["ms_stage2_kernel"]
    k1_ms = st0["ms_stage1"]
    succ = st0["rx_paths"]
    sm_mhz = clocks["sm_mhz"] or 2070.0
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = n_sm * 128 * 2 * sm_mhz * 1e6 / 1e12
    # stage 1 (the dominant kernel): algorithmic output = the reference's
    # forward records (60 B each); work = ideal-BVH flop per query
    alg1 = RECORD_BYTES * st0["fwd_records"]
    gbs1 = alg1 / (k1_ms * 1e-3) / 1e9 if k1_ms > 0 else 0.0
    tfl1 = FLOP_PER_SEGMENT_FWD * st0["segments_fwd"] / (k1_ms * 1e-3) / 1e12 if k1_ms > 0 else 0.0
    # stage 2: 32 B per verified backward ray + 64 B per task
    alg2 = 32 * succ + 64 * st0["tasks"]
    gbs2 = alg2 / (k2_ms * 1e-3) / 1e9 if k2_ms > 0 else 0.0
    tfl2 = FLOP_PER_SEGMENT * st0["segments_bwd"] / (k2_ms * 1e-3) / 1e12 if k2_ms > 0 else 0.0
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        threads = os.cpu_count() or 1
        p_, t_ = cpu_tracer_sample(cfg, threads)
        cpu = {"value": p_ / t_, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "one full coverage-128 build (C oracle, OpenMP)"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 geometry, f64 phase",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "l2": "flushed between steps (256 MB write)",
                   "rx_paths_per_step": st0["rx_paths"], "unique_paths": st0["unique_paths"],
                   "rounds": st0["rounds"], "tasks": st0["tasks"],
                   "ms_stage1": st0["ms_stage1"], "ms_stage2": st0["ms_stage2"],
                   "ms_stage2_kernel": k2_ms, "ms_bvh": st0["ms_bvh"],
                   "wall_s_timed_region": t_wall, "replicas": "one seeded scene per rank"},
        "e2e": e2e,
        "gpu_launches": kernel_launches(st0, False) * args.steps,
        "roofline": {"bound": "hbm", "kernel": "k_stage1", "achieved": gbs1, "peak": hbm,
                     "unit": "GB/s", "frac": gbs1 / hbm, "traffic": stage1_traffic(),
                     "peak_kind": peak_kind, "algorithmic_bytes": alg1,
                     "note": "forward discovery is latency/divergence bound (BVH, scene and "
                             "path table stay in L2); see roofline_alu"},
        "roofline_alu": {"bound": "fp32", "kernel": "k_stage1", "achieved": tfl1,
                         "peak": fp32_peak, "unit": "TFLOP/s", "frac": tfl1 / fp32_peak,
                         "flop_per_segment": FLOP_PER_SEGMENT_FWD,
                         "segments": st0["segments_fwd"],
                         "peak_kind": f"{n_sm} SM x 128 lanes x 2 at the sampled SM clock"},
        "roofline_stage2": {"bound": "hbm", "kernel": "k_stage2", "achieved": gbs2, "peak": hbm,
                            "unit": "GB/s", "frac": gbs2 / hbm, "traffic": stage2_traffic(),
                            "peak_kind": peak_kind, "algorithmic_bytes": alg2,
                            "acc_adds_per_verified_ray": (st0["acc_adds"] / succ if succ
                                                          else None)},
        "roofline_stage2_alu": {"bound": "fp32", "kernel": "k_stage2", "achieved": tfl2,
                                "peak": fp32_peak, "unit": "TFLOP/s", "frac": tfl2 / fp32_peak,
                                "flop_per_segment": FLOP_PER_SEGMENT,
                                "segments": st0["segments_bwd"]},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "secondary": secondary,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
