#!/usr/bin/env python
"""Benchmark of the plain method's RK4 step on one GB300 (FP64 DOF·stage/s).

Workload: N = 512 (262 144 elements), q_u = q_v = 6, source mode, constant
coefficients c = 1, α = 1e-6, β = 8, Gaussian source, bottom :absorbing_2beta
and three :wall sides with κ = 0.5, alternating flux, Chebyshev mass solver,
dt = h / (10 q²) — the GPU-scale configuration of the reference's plain method.
The state is synthetic and seeded (the reference measures on no dataset): a
steep circular front across which 1 - 2βv_h spans about [0.42, 1.58] (the
regime of data/steepening/nl; up to about 30 Chebyshev steps at the front, one
or two elsewhere), and, reported beside it, a short-wave state where every
element spans that range and the zero state (one Chebyshev step).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one RK4 step over the whole mesh (4 RHS stages). `value` is
DOF·stage/s with the state resident in HBM (CUDA events on the library's
stream); `e2e` is the same metric through the public API (Workspace.rk4_steps)
with pinned host buffers copied in and out every step. Under torchrun each
rank runs an independent replica (the path has no exchange step on one mesh).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

Q, NMESH = 6, 512
KW = dict(mixed=False, mode="source", kappa=0.5, flux="alternating",
          boundary=dict(bot="absorbing_2beta", top="wall", lft="wall", rgt="wall"))
COEF = dict(c=1.0, alpha=1e-6, beta=8.0)
T0 = 0.53
SAMPLE_N = 64          # CPU sample mesh (same degree, coefficients and sides)


def workload_name():
    return (f"plain method N={NMESH} q_u=q_v={Q} source mode, c=1 alpha=1e-6 beta=8, bottom absorbing_2beta + "
            f"3 walls kappa=0.5, alternating flux, Chebyshev, RK4 dt=h/(10q^2)")


AMP = 0.58 / (2 * COEF["beta"])   # |2βv| ≤ 0.58: 1 - 2βv_h within [0.42, 1.58]


def _project(f, N, n):
    """Modal coefficients (N, N, n, n), column-major, of the L² projection of f(x, y)."""
    from edg_westervelt_gb300.quadrature import GaussQCofs, JacobiP
    z, w = GaussQCofs(n + 2)
    P = np.stack([JacobiP(z, 0, 0, d) for d in range(n)], axis=1)
    h = 1.0 / N
    c = (np.arange(N)[:, None] + 0.5 + 0.5 * z[None, :]) * h          # [cell, point]
    X = c[None, :, None, :]                                           # [j, k, r, s]: x of column k
    Y = c[:, None, :, None]
    F = f(np.broadcast_to(X, (N, N, len(z), len(z))), np.broadcast_to(Y, (N, N, len(z), len(z))))
    return np.asfortranarray(np.einsum("ra,r,jkrs,s,sb->jkab", P, w, F, w, P, optimize=True))


def synthetic_state(N, nu, nv, seed, kind="front"):
    """Seeded smooth states, defined in units of the element size h so that every mesh sees
    the same per-element variation:
      front    v = A tanh((r - R)/h) around the source point, r = |x - (0.15, 0.5)|,
               R seeded in [0.3, 0.4]: a steepened circular front (1 - 2βv_h spans
               [0.42, 1.58] across the front, about 30 Chebyshev steps there, 1-2 elsewhere);
      uniform  v = A sin(2πx/h) sin(2π y/h + φ): every element spans the whole range;
      zero     u = v = 0.
    u is 1e-4 times a smooth seeded field in all but the zero state."""
    rng = np.random.default_rng(seed)
    if kind == "zero":
        return np.zeros((N, N, nu, nu), order="F"), np.zeros((N, N, nv, nv), order="F")
    h = 1.0 / N
    a, b = rng.uniform(1, 3, 2)
    u = _project(lambda x, y: 1e-4 * np.sin(a * np.pi * x) * np.cos(b * np.pi * y), N, nu)
    if kind == "front":
        R = rng.uniform(0.3, 0.4)
        v = _project(lambda x, y: AMP * np.tanh((np.hypot(x - 0.15, y - 0.5) - R) / h), N, nv)
    else:
        ph = rng.uniform(0, 2 * np.pi)
        v = _project(lambda x, y: AMP * np.sin(2 * np.pi * x / h) * np.sin(2 * np.pi * y / h + ph), N, nv)
    return u, v


def alg_bytes_per_element_stage(nu, nv, qh, one_sided=False, s_mode_nv2=1):
    """Algorithmic bytes of one element in one RK4 stage (reference data model, FP64)."""
    nq = nu
    return 8 * (nu * nu * (nu * nu + 1) / 2 + 2 * nu * nu + qh * qh + 8 * nq + (6 * nq if one_sided else 0)
                + s_mode_nv2 * nv * nv + 4.25 * (nu * nu + nv * nv))


def alg_flops_per_element_stage(nu, nv, qh, n_cheb):
    nq = nu
    f = (16 * nu ** 3 + 8 * nu * nv * (nu + nv) + 2 * nu ** 4 + 16 * nu ** 2 + 16 * nv ** 2 + 16 * nu * nv
         + 4 * (4 * nv * nq + 2 * nu * nq + 4 * nv * nv + 2 * nu * nu) + 60 * nq + 2 * qh * nv * (nv + qh)
         + 2 * (nu * nu + nv * nv))
    return f + (n_cheb - 1) * (4 * qh * nv * (nv + qh) + 10 * nv * nv)


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, power, throttle reasons)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
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
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["not sampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 4 + i and r[4 + i] == "Active"})
        power = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w_max": max(power) if power else None, "samples": len(self.rows), "reasons": reasons}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        return {}


def fp64_gemm_peak(torch, dev):
    """cuBLAS DGEMM throughput (TFLOP/s), the FP64 denominator: best of 3, n = 4096."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    return 2 * n ** 3 / best / 1e12


def profile_figures():
    """DRAM bytes per RHS stage and the FP64-pipe utilisation of each stage kernel, from the
    committed ncu summary of the stage kernels (None where it is missing)."""
    p = os.path.join(ROOT, "profiles", "stage_dram_N512_q6.txt")
    out = {"traffic": None, "fp64_pipe_pct": {}}
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_stage:"):
                out["traffic"] = float(line.split(":")[1])
            elif line.startswith("fp64_pipe_pct "):
                k, v = line[len("fp64_pipe_pct "):].split(":")
                out["fp64_pipe_pct"][k.strip()] = float(v)
    except OSError:
        pass
    return out


def bench_config(E, dof, state):
    """The `config` of the bench line, the same for the GPU arm and the reference arm (the
    algorithmic choices of each arm, e.g. its Chebyshev step policy, are reported outside it)."""
    return {"workload": workload_name(), "elements": E, "dof": dof,
            "state": {"front": "steepened circular front, 1-2βv_h in [0.42, 1.58] across it (seeded)",
                      "uniform": "short-wave state, every element spans 1-2βv_h in [0.42, 1.58] (seeded)",
                      "zero": "zero state"}[state],
            "l2": "inputs larger than L2 (state 206 MB, stage data > 600 MB per stage)", "t0": T0}


class CpuPort:
    """The oracle (C restatement of the reference's RHS and RK4, OpenMP on all host threads)
    on the same configuration at mesh N, from the oracle's own precompute, on the GPU arm's
    seeded state (seed 0)."""

    def __init__(self, N, kind="front"):
        from oracle import coefficients as oc
        from oracle.precompute import precompute as opre
        from oracle.rhs import OracleWorkspace, max_threads
        t0 = time.perf_counter()
        pre, _ = opre(Q, N, coefficients=oc.constant_coefficients(**COEF), **KW)
        self.setup_s = time.perf_counter() - t0
        self.u, self.v = synthetic_state(N, pre["qu1"], pre["qv1"], seed=0, kind=kind)
        self.ws = OracleWorkspace(pre)
        self.dt = (1.0 / N) / (10 * Q * Q)
        self.dof = N * N * (pre["qu1"] ** 2 + pre["qv1"] ** 2)
        self.cores = max_threads()
        self.n = 0

    def step(self):
        t0 = time.perf_counter()
        self.ws.rk4_step(self.u, self.v, T0 + self.n * self.dt, self.dt)
        self.n += 1
        return time.perf_counter() - t0


def cpu_baseline(budget_s):
    port = CpuPort(SAMPLE_N)
    port.step()
    n, t = 0, 0.0
    while (n < 2 or t < budget_s) and n < 200:
        t += port.step()
        n += 1
    return port.dof * 4 * n / t, n, t, port.cores


def max_over_ranks(x, dist, device):
    """The largest of the ranks' values of x (the slowest replica sets the whole job's time)."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(dof_per_rank, world, steps, ms_max):
    """Whole-job DOF·stage/s of `world` replicas, each advancing dof_per_rank DOF by `steps` RK4
    steps, over the slowest rank's time in milliseconds."""
    return world * dof_per_rank * 4 * steps / (ms_max / 1e3)


def run_reference(args):
    """The reference's CPU path on the host cores: the oracle port (Julia is not installed), on
    the GPU arm's workload -- the same mesh, degrees, coefficients, sides, flux and seeded state --
    with the reference's algorithm (every element takes the common maximum Chebyshev count,
    src/rhs.jl:911-918, and the stored inverse stiffnesses)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    port = CpuPort(NMESH, kind=args.state)
    for _ in range(args.warmup):
        port.step()
    t = sum(port.step() for _ in range(args.steps))
    value = port.dof * 4 * args.steps / t
    E = NMESH * NMESH
    sample = (f"{args.steps} RK4 steps (after {args.warmup} warm-up) of the full workload (N={NMESH}, {E} "
              f"elements, the GPU arm's seeded state); oracle precompute {port.setup_s:.0f} s, not timed")
    line = {"impl": "reference", "metric": "FP64 DOF·stage/s on 1 GB300 (plain method, RK4 step)", "value": value,
            "unit": "DOF·stage/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded state)",
            "config": bench_config(E, port.dof, args.state),
            "algorithm": {"cheb_steps": "common maximum over the elements (src/rhs.jl:911-918)",
                          "u_solve": "stored packed inverse stiffnesses (src/rhs.jl:352-382)"},
            "cpu_baseline": {"value": value, "unit": "DOF·stage/s", "cores": port.cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "DOF·stage/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "Julia (the reference's toolchain) is not installed here or on the GPU box; the timed CPU path "
                    "is the oracle's C restatement of src/rhs.jl + src/solver.jl with OpenMP on all host threads"}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import edg_westervelt_gb300 as W

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", init_method="env://")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if args.batched_only:
        print(json.dumps({"batched": run_batched(torch, dev, args.steps, args.warmup)}), flush=True)
        return
    if args.adjoint:
        print(json.dumps({"adjoint": run_adjoint(torch, args.adjoint_T, args.adjoint_every, args.adjoint_batch,
                                                 args.adjoint_batch_T)}), flush=True)
        return
    if args.general_only:
        print(json.dumps({"general": run_general(torch, dev, args.steps, args.warmup)}), flush=True)
        return

    t_setup = time.perf_counter()
    pre, _ = W.precompute(Q, NMESH, coefficients=W.constant_coefficients(**COEF), target="device", **KW)
    N, nu, nv, qh = NMESH, pre["qu1"], pre["qv1"], pre["q_high"]
    E = N * N
    dof = E * (nu * nu + nv * nv)
    dt = (1.0 / N) / (10 * Q * Q)
    ws = W.Workspace(pre, N)
    t_setup = time.perf_counter() - t_setup
    t_host = time.perf_counter()
    pre_host, _ = W.precompute(Q, NMESH, coefficients=W.constant_coefficients(**COEF), **KW)
    W.Workspace(pre_host, N)
    t_host = time.perf_counter() - t_host
    del pre_host

    def device_state(kind, seed):
        u, v = synthetic_state(N, nu, nv, seed, kind)
        # the reference's column-major bytes, as flat device tensors
        return (torch.from_numpy(u.reshape(-1, order="F").copy()).to(dev),
                torch.from_numpy(v.reshape(-1, order="F").copy()).to(dev))

    def timed(kind, steps, warmup, ws=ws):
        u, v = device_state(kind, seed=0)
        u0, v0 = u.clone(), v.clone()
        lib = __import__("edg_westervelt_gb300._lib", fromlist=["lib"]).lib()
        import ctypes
        up, vp = ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(v.data_ptr())
        torch.cuda.synchronize()
        rc = lib.wedg_rk4_steps_async(ws._h, up, vp, T0, dt, warmup)
        ws._check(lib.wedg_sync_status(ws._h, None, None) if rc == 0 else rc)
        u.copy_(u0)
        v.copy_(v0)
        lib.wedg_time_kernels(ws._h, 1)
        lib.wedg_kernel_times(ws._h, None, None, None, None, None, None, 1)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ext = torch.cuda.ExternalStream(ws.stream, device=dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(ext):
            e0.record(ext)
        rc = lib.wedg_rk4_steps_async(ws._h, up, vp, T0, dt, steps)
        launches = ws.stats()["kernel_launches"]
        with torch.cuda.stream(ext):
            e1.record(ext)
        done = ctypes.c_int64(0)
        ws._check(lib.wedg_sync_status(ws._h, ctypes.byref(done), None) if rc == 0 else rc)
        torch.cuda.synchronize()
        if done.value != steps:
            raise RuntimeError(f"only {done.value} of the {steps} timed RK4 steps completed")
        ms = e0.elapsed_time(e1)
        if dist:
            ms = max_over_ranks(ms, dist, dev)
            dist.barrier()
        pm, pn, sm, sn = (ctypes.c_double(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_int64())
        mm, mn = ctypes.c_double(), ctypes.c_int64()
        lib.wedg_kernel_times(ws._h, ctypes.byref(pm), ctypes.byref(pn), ctypes.byref(sm), ctypes.byref(sn),
                              ctypes.byref(mm), ctypes.byref(mn), 1)
        lib.wedg_time_kernels(ws._h, 0)
        st = ws.stats()
        return dict(ms=ms, steps=int(done.value), launches=launches, prep_ms=pm.value / max(pn.value, 1),
                    stage_ms=sm.value / max(sn.value, 1), n_stage=sn.value, cheb=st["cheb_steps_max"],
                    mass_ms=mm.value / max(mn.value, 1),
                    cheb_mean=st["cheb_steps_sum"] / max(st["element_stages"], 1))

    with ClockSampler(local) as clocks:
        main = timed(args.state, args.steps, args.warmup)
    if args.profile_only:
        return
    zero = timed("zero", max(2, args.steps // 4), args.warmup)
    unif = timed("uniform", max(2, args.steps // 4), args.warmup)
    # the reference's own Chebyshev policy (every element takes the largest count of the stage,
    # src/rhs.jl:911-918) on the same state: the same algorithm as the reference arm
    ws_common = W.Workspace(pre, N, cheb_steps="common_max")
    common = timed(args.state, args.steps, args.warmup, ws=ws_common)
    del ws_common

    ms_step = main["ms"] / args.steps
    value = replica_value(dof, world, args.steps, main["ms"])

    # one edg_rhs! per call (wedg_rhs on device-resident state, each call returning synchronised
    # with its error word read): the per-evaluation time of the RHS alone, at the front state
    # advanced by `warmup` RK4 steps (the exact initial projection has nearly constant v on the
    # elements away from the front, one Chebyshev step each; a few steps give them the counts
    # they keep along the run)
    ur, vr = device_state(args.state, seed=0)
    utr, vtr = torch.empty_like(ur), torch.empty_like(vr)
    t_r = T0 + max(args.warmup, 1) * dt
    if ws.rk4_steps(ur, vr, T0, dt, max(args.warmup, 1)) != max(args.warmup, 1):
        raise RuntimeError("the RK4 steps before the edg_rhs! timing did not complete")
    for _ in range(args.warmup):
        ws.rhs(ur, vr, t_r, utr, vtr)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ws.rhs(ur, vr, t_r, utr, vtr)
    t_rhs = (time.perf_counter() - t0) / args.steps
    rhs_call = {"ms_per_call": t_rhs * 1e3, "value": world * dof / t_rhs, "unit": "DOF·stage/s",
                "calls": args.steps, "cheb_steps_max": ws.stats()["cheb_steps_max"],
                "cheb_steps_mean": ws.stats()["cheb_steps_sum"] / max(ws.stats()["element_stages"], 1),
                "timing": "host clock around each call (wedg_rhs with device pointers: three kernels, the "
                          "error word read back, synchronised); the front state after the warm-up's RK4 steps"}
    del ur, vr, utr, vtr

    # end to end through the public API: pinned host state in, result out, every step
    e2e = None
    if rank == 0 or world > 1:
        tu = torch.empty(E * nu * nu, dtype=torch.float64, pin_memory=True)
        tv = torch.empty(E * nv * nv, dtype=torch.float64, pin_memory=True)
        uh = tu.numpy().reshape((N, N, nu, nu), order="F")
        vh = tv.numpy().reshape((N, N, nv, nv), order="F")
        us, vs = synthetic_state(N, nu, nv, 0, "front")
        uh[...] = us
        vh[...] = vs
        ws.rk4_steps(uh, vh, T0, dt, 1)               # warm-up
        uh[...] = us
        vh[...] = vs
        ke = args.steps
        t0 = time.perf_counter()
        for i in range(ke):
            if ws.rk4_steps(uh, vh, T0 + i * dt, dt, 1) != 1:
                raise RuntimeError("an end-to-end RK4 step did not complete")
        te = time.perf_counter() - t0
        e2e = {"value": world * dof * 4 * ke / te, "unit": "DOF·stage/s",
               "h2d_bytes_per_step": int(uh.nbytes + vh.nbytes), "d2h_bytes_per_step": int(uh.nbytes + vh.nbytes),
               "steps": ke, "api": "Workspace.rk4_steps (wedg_rk4_steps, WEDG_HOST)"}

    batched = config3 = general = adjoint = None
    if world == 1 and not args.no_batched:
        batched = run_batched(torch, dev, max(4, 2 * args.steps), args.warmup)
        config3 = run_config3(torch, dev, args.steps, args.warmup)
        general = run_general(torch, dev, args.steps, args.warmup)
    if world == 1 and not args.no_adjoint:
        adjoint = run_adjoint(torch, args.adjoint_T, args.adjoint_every, args.adjoint_batch, args.adjoint_batch_T)

    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    bytes_stage = alg_bytes_per_element_stage(nu, nv, qh) * E
    kms = {"k_prep": main["prep_ms"], "k_stage": main["stage_ms"], "k_cheb": main["mass_ms"]}
    stage_ms = sum(kms.values())
    dominant = max(kms, key=kms.get)
    achieved_gbs = bytes_stage / (stage_ms / 1e3) / 1e9
    fp64_peak = fp64_gemm_peak(torch, dev)
    # algorithmic flops of the stage with every element's own Chebyshev count (mean from the device counter)
    f1 = alg_flops_per_element_stage(nu, nv, qh, 1)
    per_step = alg_flops_per_element_stage(nu, nv, qh, 2) - f1
    flops_stage = (f1 + (main["cheb_mean"] - 1) * per_step) * E
    fp64_achieved = flops_stage / (stage_ms / 1e3) / 1e12
    prof = profile_figures()
    roofline = {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm, "unit": "GB/s",
                "frac": achieved_gbs / hbm if hbm else None, "traffic": prof["traffic"],
                "kernel": "RHS stage (k_prep + k_stage + k_cheb)", "dominant_kernel": dominant,
                "dominant_share": kms[dominant] / stage_ms, "bytes_per_launch": bytes_stage, "launch_ms": stage_ms,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if hbm else None,
                "note": "the stage is bound by the FP64 pipe, not by HBM (see fp64_pipe); bytes are the "
                        "reference data model's algorithmic bytes per element-stage x elements, over the time "
                        "of one RHS stage (its three kernels); traffic is ncu's DRAM bytes of the three kernels "
                        "per stage (profiles/stage_dram_N512_q6.txt)"}
    pipe = prof["fp64_pipe_pct"]
    fp64_pipe = None
    if pipe and all(k in pipe for k in kms):
        fp64_pipe = {"unit": "% of the FP64 pipe's peak sustained rate over active cycles (ncu)",
                     "per_kernel": pipe,
                     "stage_weighted": sum(pipe[k] * kms[k] for k in kms) / stage_ms,
                     "source": "profiles/stage_kernels_N256_q6.md"}
    reference_ops = {"value": fp64_achieved, "unit": "TFLOP/s", "dgemm_peak": fp64_peak,
                     "flops_per_stage": flops_stage,
                     "cheb_steps_max": main["cheb"], "cheb_steps_mean": main["cheb_mean"],
                     "peak_source": "cuBLAS DGEMM 4096^3 measured in this run",
                     "note": "the reference's FP64 operation count of a stage (each element's own Chebyshev "
                             "count) over the k_prep + k_stage + k_cheb time; it can exceed the DGEMM rate "
                             "because the kernels execute fewer FP64 operations than that count (mirror "
                             "parity of the Gauss-Legendre rules, fast diagonalisation of the u-equation, "
                             "constant-coefficient volume terms)"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        r, n, t, cores = cpu_baseline(args.cpu_seconds)
        cpu = {"value": r, "unit": "DOF·stage/s", "cores": cores, "kind": "port",
               "sample": f"{n} RK4 steps ({t:.1f} s) of the same configuration and front state on an N={SAMPLE_N} "
                         f"mesh; the oracle's C restatement with OpenMP"}
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    line = {
        "metric": "FP64 DOF·stage/s on 1 GB300 (plain method, RK4 step)", "value": value, "unit": "DOF·stage/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded steepened-wave state; the reference measures on no dataset)",
        "config": bench_config(E, dof, args.state),
        "algorithm": {"cheb_steps": "per element: each element takes the count its own spectral interval "
                                    "needs for the reference's tolerance (the reference's common maximum is "
                                    "in common_max)",
                      "u_solve": "fast diagonalisation of the constant-coefficient stiffness"},
        "common_max": {"value": world * dof * 4 * common["steps"] / (common["ms"] / 1e3),
                       "ms_per_step": common["ms"] / max(common["steps"], 1), "cheb_steps_max": common["cheb"],
                       "stage_ms": common["prep_ms"] + common["stage_ms"] + common["mass_ms"],
                       "note": "the same workload and state with the reference's Chebyshev policy: every element "
                               "takes the stage's largest count (src/rhs.jl:911-918), as the reference arm does"},
        "rhs_call": rhs_call,
        "roofline": roofline, "fp64_pipe": fp64_pipe, "reference_op_rate": reference_ops,
        "cpu_baseline": cpu, "e2e": e2e,
        "clocks": clocks.summary(), "gpu_launches": main["launches"],
        "kernel_ms": kms,
        "setup_s": {"device_built_pre": t_setup, "host_pre": t_host,
                    "note": "precompute + Workspace: pre's large arrays built on the device from the coefficients' "
                            "values (precompute(target='device'), wedg_create_points) against the host precompute"},
        "batched": batched,
        "adjoint": adjoint,
        "config3": config3,
        "general": general,
        "zero_state": {"value": world * dof * 4 * zero["steps"] / (zero["ms"] / 1e3),
                       "ms_per_step": zero["ms"] / max(zero["steps"], 1), "cheb_steps_max": zero["cheb"],
                       "stage_ms": zero["prep_ms"] + zero["stage_ms"] + zero["mass_ms"]},
        "uniform_state": {"value": world * dof * 4 * unif["steps"] / (unif["ms"] / 1e3),
                          "ms_per_step": unif["ms"] / max(unif["steps"], 1), "cheb_steps_max": unif["cheb"],
                          "stage_ms": unif["prep_ms"] + unif["stage_ms"] + unif["mass_ms"],
                          "note": "every element spans 1-2βv in [0.42, 1.58]: no element is cheap"},
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


BATCH_SIZES = (16, 24, 32, 48, 64, 96, 128)


def batch_instances(n=256, seed=4):
    """The mixed batch: n instances drawn from default_rng(seed): N from BATCH_SIZES, q_u from
    2..7, q_v in {q_u - 1, q_u}, flux and the four boundary kinds uniformly, and c ~ U[0.5, 2],
    α log-uniform on [1e-6, 1e-3], β ~ U[0, 10] constant on each of 4 × 4 mesh-aligned
    subsquares; source mode (Gaussian source) from the zero state, dt = h / (dt_fac q_u²) with
    dt_fac = 10 max c. Yields (q_u, N, precompute keywords, dt)."""
    import edg_westervelt_gb300 as W
    rng = np.random.default_rng(seed)

    for _ in range(n):
        N = int(rng.choice(BATCH_SIZES))
        qu = int(rng.integers(2, 8))
        qv = int(rng.choice([qu - 1, qu]))
        flux = str(rng.choice(["upwind", "central", "alternating"]))
        kinds = [str(k) for k in rng.choice(["absorbing_2beta", "absorbing", "dirichlet", "wall"], 4)]
        c = rng.uniform(0.5, 2.0, (4, 4))
        al = 10.0 ** rng.uniform(-6, -3, (4, 4))
        be = rng.uniform(0.0, 10.0, (4, 4))
        co = W.cell_coefficients(c, al, be)
        kw = dict(mixed=(qv == qu - 1), flux=flux, mode="source", coefficients=co, kappa=0.5,
                  boundary=dict(bot=kinds[0], top=kinds[1], lft=kinds[2], rgt=kinds[3]))
        yield qu, N, kw, (1.0 / N) / (10.0 * float(c.max()) * qu * qu)


def run_batched(torch, dev, steps, warmup):
    """The batched form against the plain per-instance loop on the same instances: aggregate
    DOF·stage/s of Batch.rk4_steps (one CUDA-graph replay per step of all instances) and of
    Workspace.rk4_steps called instance after instance, both on device-resident states."""
    import edg_westervelt_gb300 as W
    t_setup = time.perf_counter()
    wss, us, vs, dts, dof = [], [], [], [], 0
    for qu, N, kw, dt in batch_instances():
        pre, _ = W.precompute(qu, N, target="device", **kw)
        ws = W.Workspace(pre, N)
        wss.append(ws)
        us.append(torch.zeros(N * N * pre["qu1"] ** 2, dtype=torch.float64, device=dev))
        vs.append(torch.zeros(N * N * pre["qv1"] ** 2, dtype=torch.float64, device=dev))
        dts.append(dt)
        dof += N * N * (pre["qu1"] ** 2 + pre["qv1"] ** 2)
    t_setup = time.perf_counter() - t_setup
    batch = W.Batch(wss)
    n = len(wss)
    t = [0.0] * n

    def advance(k):
        for i in range(n):
            t[i] += k * dts[i]
    batch.rk4_steps(us, vs, t, dts, warmup)                       # captures the graph
    advance(warmup)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    done, fin, _ = batch.rk4_steps(us, vs, t, dts, steps)
    tb_default = time.perf_counter() - t0
    advance(steps)
    assert all(d == steps for d in done) and all(fin)
    # the autotuner: launch shapes per bucket, on copies of the present states
    shapes_default = [dict(s) for s in batch.shapes()]
    t0 = time.perf_counter()
    ms_tuner = batch.autotune(us, vs, t, dts, steps=2)
    t_tune = time.perf_counter() - t0
    shapes = [dict(s) for s in batch.shapes()]
    batch.rk4_steps(us, vs, t, dts, 1)                            # captures the tuned graph
    advance(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    done, fin, _ = batch.rk4_steps(us, vs, t, dts, steps)
    tb = time.perf_counter() - t0
    advance(steps)
    assert all(d == steps for d in done) and all(fin)
    for i, ws in enumerate(wss):                                  # warm the single-instance path
        ws.rk4_steps(us[i], vs[i], t[i], dts[i], 1)
    advance(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i, ws in enumerate(wss):
        assert ws.rk4_steps(us[i], vs[i], t[i], dts[i], steps) == steps
    tp = time.perf_counter() - t0
    tbest = min(tb, tb_default)
    vb, vp = dof * 4 * steps / tbest, dof * 4 * steps / tp
    return {"workload": "256 instances, N in {16..128}, q_u 2-7, q_v in {q_u-1, q_u}, random flux and boundary "
                        "kinds, piecewise-constant c, alpha, beta on 4x4 subsquares (default_rng(4)), source mode",
            "instances": n, "buckets": len(shapes), "elements": int(sum(w.N * w.N for w in wss)), "dof": int(dof),
            "steps": steps, "value": vb, "unit": "DOF·stage/s", "ms_per_step": tbest / steps * 1e3,
            "plain_loop_value": vp, "plain_loop_ms_per_step": tp / steps * 1e3, "speedup_vs_plain_loop": vb / vp,
            "setup_s": t_setup,
            "autotune": {"default_ms_per_step": tb_default / steps * 1e3, "tuned_ms_per_step": tb / steps * 1e3,
                         "tuner_median_ms_per_step": ms_tuner, "tune_s": t_tune, "shapes": shapes,
                         "kept_default_shapes": shapes == shapes_default,
                         "note": "per bucket: the layout (persist -1: the instances' own launches; 0: one launch per "
                                 "stage kernel over the bucket; > 0: persistent grids) and the threads per block of "
                                 "k_prep and of the mass solves (Batch.autotune, paired trials; kept only on a 2 % "
                                 "gain of the whole batch); value and ms_per_step are the faster of the default-shape "
                                 "and the tuned-shape runs (the same shapes when kept_default_shapes); both are "
                                 "reported here"},
            "timing": "host clock around each call (each call returns synchronised); states resident on the GPU",
            "batched": "Batch.rk4_steps: buckets of instances with the same kernels side by side, each bucket's "
                       "instances on their own streams (the default) or one multi-instance launch per stage kernel "
                       "(the tuner's choice per bucket); CUDA graphs of one and of four RK4 steps of every instance, "
                       "replayed",
            "plain_loop": "Workspace.rk4_steps for each instance in turn"}


def device_steps_ms(torch, ws, u, v, t0, dt, steps, warmup):
    """Milliseconds of `steps` RK4 steps on device-resident states after `warmup` untimed ones (CUDA
    events on the workspace's stream around wedg_rk4_steps_async)."""
    import ctypes
    from edg_westervelt_gb300 import _lib as L
    lib = L.lib()
    up, vp = ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(v.data_ptr())
    ext = torch.cuda.ExternalStream(ws.stream, device=u.device)
    rc = lib.wedg_rk4_steps_async(ws._h, up, vp, t0, dt, warmup)
    ws._check(lib.wedg_sync_status(ws._h, None, None) if rc == 0 else rc)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(ext):
        e0.record(ext)
    rc = lib.wedg_rk4_steps_async(ws._h, up, vp, t0 + warmup * dt, dt, steps)
    with torch.cuda.stream(ext):
        e1.record(ext)
    ws._check(lib.wedg_sync_status(ws._h, None, None) if rc == 0 else rc)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def run_general(torch, dev, steps, warmup):
    """The headline workload with smoothly varying coefficients, so that the general kernels run
    (per-element quadrature coefficients Cw, Aw and the packed inverse stiffness Ainv, the
    reference's dominant byte stream): c = 1 + 0.1 cos(πx) cos(πy), α = 1e-6 (1 + 0.1 cos(πx)
    cos(πy)), β = 8 (1 + 0.1 sin(πx) sin(πy)); N = 512, q = 6, the same sides, flux and steep
    front state. DOF·stage/s, the stage kernels' times and the algorithmic HBM rate."""
    import ctypes
    import math
    import edg_westervelt_gb300 as W
    from edg_westervelt_gb300 import _lib as L
    pi = math.pi
    cc = lambda x, y: np.cos(pi * x) * np.cos(pi * y)
    ss = lambda x, y: np.sin(pi * x) * np.sin(pi * y)
    co = W.Coefficients(lambda x, y: 1 + 0.1 * cc(x, y),
                        lambda x, y: -0.1 * pi * np.sin(pi * x) * np.cos(pi * y),
                        lambda x, y: -0.1 * pi * np.cos(pi * x) * np.sin(pi * y),
                        lambda x, y: 1e-6 * (1 + 0.1 * cc(x, y)),
                        lambda x, y: -1e-7 * pi * np.sin(pi * x) * np.cos(pi * y),
                        lambda x, y: -1e-7 * pi * np.cos(pi * x) * np.sin(pi * y),
                        lambda x, y: 8.0 * (1 + 0.1 * ss(x, y)))
    N = NMESH
    t0 = time.perf_counter()
    pre, _ = W.precompute(Q, N, coefficients=co, target="device", **KW)
    ws = W.Workspace(pre, N)
    setup_s = time.perf_counter() - t0
    nu, nv, qh = pre["qu1"], pre["qv1"], pre["q_high"]
    E = N * N
    us, vs = synthetic_state(N, nu, nv, 0, "front")
    u = torch.from_numpy(us.reshape(-1, order="F").copy()).to(dev)
    v = torch.from_numpy(vs.reshape(-1, order="F").copy()).to(dev)
    dt = (1.0 / N) / (10 * Q * Q)
    lib = L.lib()
    lib.wedg_time_kernels(ws._h, 1)
    lib.wedg_kernel_times(ws._h, None, None, None, None, None, None, 1)
    ms = device_steps_ms(torch, ws, u, v, T0, dt, steps, warmup)
    pm, pn, sm, sn = (ctypes.c_double(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_int64())
    mm, mn = ctypes.c_double(), ctypes.c_int64()
    lib.wedg_kernel_times(ws._h, ctypes.byref(pm), ctypes.byref(pn), ctypes.byref(sm), ctypes.byref(sn),
                          ctypes.byref(mm), ctypes.byref(mn), 1)
    lib.wedg_time_kernels(ws._h, 0)
    kms = {"k_prep": pm.value / max(pn.value, 1), "k_stage": sm.value / max(sn.value, 1),
           "k_cheb": mm.value / max(mn.value, 1)}
    stage_ms = sum(kms.values())
    dof = E * (nu * nu + nv * nv)
    bytes_stage = alg_bytes_per_element_stage(nu, nv, qh) * E
    return {"workload": f"general kernels: N={N} q_u=q_v={Q}, source mode, c, alpha, beta varying by 10 % "
                        "(cos/sin in x, y) around c=1, alpha=1e-6, beta=8; same sides, flux and front state",
            "value": dof * 4 * steps / (ms / 1e3), "unit": "DOF·stage/s", "ms_per_step": ms / steps,
            "steps": steps, "fast_path": bool(ws.stats()["fast_path"]), "setup_s": setup_s,
            "kernel_ms": kms, "stage_alg_gbs": bytes_stage / (stage_ms / 1e3) / 1e9,
            "note": "timing covers all warm-up and timed steps' kernels; stage_alg_gbs = the reference data "
                    "model's bytes of one stage over the three stage kernels' mean time"}


def config3_problem(precompute=None):
    """The jumping-coefficient workload: N = 256, q_u = 5, q_v = 4, initial-value mode, c, α, β
    constant on 4 × 4 subsquares from default_rng(3) (c ~ U[0.5, 2], α log-uniform on [1e-6, 1e-3],
    β ~ U[0, 10]), initial displacement a sum of 3 seeded Gaussians (centres U[0.2, 0.8]², widths
    U[0.03, 0.08], amplitudes U[-1, 1] scaled to 1e-3 so that 1 - 2βv stays positive), sides
    dirichlet / absorbing / absorbing_2beta / wall (bot, top, lft, rgt), central flux, one-sided faces,
    dt = h / (10 max c q_u²). Returns (pre, N, dt) from `precompute` (default the package's)."""
    import edg_westervelt_gb300 as W
    precompute = precompute or W.precompute
    rng = np.random.default_rng(3)
    q, N = 5, 256
    c = rng.uniform(0.5, 2.0, (4, 4))
    al = 10.0 ** rng.uniform(-6, -3, (4, 4))
    be = rng.uniform(0.0, 10.0, (4, 4))
    cen = rng.uniform(0.2, 0.8, (3, 2))
    wid = rng.uniform(0.03, 0.08, 3)
    amp = 1e-3 * rng.uniform(-1.0, 1.0, 3)

    def gauss(d):
        def f(x, y):
            x = np.asarray(x, dtype=float)
            y = np.asarray(y, dtype=float)
            out = np.zeros(np.broadcast(x, y).shape)
            for (x0, y0), w, a in zip(cen, wid, amp):
                X, Y = x - x0, y - y0
                gv = a * np.exp(-(X * X + Y * Y) / (w * w))
                out = out + {"": gv, "x": -2 * X / w ** 2 * gv, "y": -2 * Y / w ** 2 * gv,
                             "xx": (4 * X * X / w ** 4 - 2 / w ** 2) * gv, "yy": (4 * Y * Y / w ** 4 - 2 / w ** 2) * gv}[d]
            return out
        return f
    prof = dict(u0=gauss(""), u0_x=gauss("x"), u0_y=gauss("y"), u0_xx=gauss("xx"), u0_yy=gauss("yy"))
    co = W.piecewise_coefficients(c ** 2, al, be)
    pre, _ = precompute(q, N, mixed=True, mode="initial_value", flux="central", coefficients=co,
                        initial_profile=prof, kappa=0.5,
                        boundary=dict(bot="dirichlet", top="absorbing", lft="absorbing_2beta", rgt="wall"))
    return pre, N, (1.0 / N) / (10.0 * float(c.max()) * q * q)


def run_config3(torch, dev, steps, warmup):
    """Plain method with jumping coefficients (config3_problem), from the reference's zero start;
    DOF·stage/s over the timed steps."""
    import edg_westervelt_gb300 as W
    pre, N, dt = config3_problem()
    ws = W.Workspace(pre, N)
    nu, nv = pre["qu1"], pre["qv1"]
    u = torch.zeros(N * N * nu * nu, dtype=torch.float64, device=dev)
    v = torch.zeros(N * N * nv * nv, dtype=torch.float64, device=dev)
    ms = device_steps_ms(torch, ws, u, v, 0.0, dt, steps, warmup)
    dof = N * N * (nu * nu + nv * nv)
    return {"workload": "plain method, jumping coefficients: N=256 q_u=5 q_v=4, initial-value mode, central flux, "
                        "4x4 subsquares of c, alpha, beta (default_rng(3)), mixed boundary kinds",
            "value": dof * 4 * steps / (ms / 1e3), "unit": "DOF·stage/s", "ms_per_step": ms / steps, "steps": steps,
            "dof": dof, "one_sided": bool(pre["one_sided"]), "fast_path": bool(ws.stats()["fast_path"])}


def adjoint_problem(seed=5, m=16):
    """The adjoint form's workload: c², α, β constant on m × m cells (c ~ U[0.8, 1.25], α log-uniform on
    [1e-6, 1e-5] -- larger α makes the explicit RK4 step unstable at this dt -- β ~ U[0, 4]) from
    default_rng(seed), a 32 × 32 receiver grid at the cell centres, forward N = 128, q_u = q_v = 4,
    absorbing_2beta sides, upwind flux, Gaussian source. Returns (rng, fields, receivers, kw)."""
    rng = np.random.default_rng(seed)
    c2 = rng.uniform(0.8, 1.25, (m, m)) ** 2
    al = 10.0 ** rng.uniform(-6, -5, (m, m))
    be = rng.uniform(0.0, 4.0, (m, m))
    g = (np.arange(32) + 0.5) / 32
    receivers = [(x, y) for y in g for x in g]
    return rng, (c2, al, be), receivers, dict(flux="upwind", mixed=False, boundary="absorbing_2beta")


def run_adjoint(torch, T, every=32, batch=16, batch_T=0.125):
    """The adjoint form (N = 128, q = 4): the gradient of J = ½ Σ_r (u_h(x_r, T) - u_obs_r)² with respect to
    the 3 × 16 × 16 cell values (adjoint_problem), u_obs from the forward solver on the field
    perturbed by ±10 %, checkpoints every 32 steps. Timed: one forward solve (Workspace.rk4_steps),
    one gradient (misfit_gradient: forward with checkpoints, misfit, reverse sweep with the parameter
    sensitivities, cell sums) and a batch of `batch` gradients for different seeded fields at once
    (misfit_gradients: every stage of all of them as multi-instance launches) over batch_T."""
    import edg_westervelt_gb300 as W
    from edg_westervelt_gb300.solver import _locate, _vrow
    q, N = 4, 128
    rng, (c2, al, be), receivers, kw = adjoint_problem()
    pert = lambda a: a * (1.0 + 0.1 * rng.uniform(-1, 1, a.shape))   # noqa: E731
    pre, _ = W.precompute(q, N, mode="source", coefficients=W.piecewise_coefficients(pert(c2), pert(al), pert(be)),
                          **kw)
    dt = (1.0 / N) / (10 * q * q)
    nsteps = int(round(T / dt))
    dt = T / nsteps
    ws = W.Workspace(pre, N)
    u = np.zeros((N, N, 5, 5), order="F")
    v = np.zeros((N, N, 5, 5), order="F")
    ws.rk4_steps(u, v, 0.0, dt, nsteps)
    u_obs = []
    for xr, yr in receivers:
        kr, xi = _locate(xr, N)
        jr, eta = _locate(yr, N)
        u_obs.append(float(_vrow(eta, 5) @ u[jr - 1, kr - 1] @ _vrow(xi, 5)))
    del ws
    # one forward solve of the unperturbed field (the step loop, host state in and out)
    pre, _ = W.precompute(q, N, mode="source", coefficients=W.piecewise_coefficients(c2, al, be), **kw)
    ws = W.Workspace(pre, N)
    u[...] = 0.0
    v[...] = 0.0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ws.rk4_steps(u, v, 0.0, dt, nsteps)
    t_fwd = time.perf_counter() - t0
    del ws
    t0 = time.perf_counter()
    J, grad = W.misfit_gradient(q, N, T, c2, al, be, receivers, u_obs, every=every, **kw)
    t_grad = time.perf_counter() - t0
    out = {"workload": f"misfit gradient, N={N} q_u=q_v={q}, 16x16 cells of c2, alpha, beta, 32x32 receivers, "
                       f"absorbing_2beta, Gaussian source, T={T} ({nsteps} RK4 steps), checkpoints every {every}",
           "value": t_grad, "unit": "s/grad", "forward_s": t_fwd, "grad_over_forward": t_grad / t_fwd,
           "misfit": J, "grad_norms": {k: float(np.linalg.norm(vv)) for k, vv in grad.items()},
           "timing": "host clock around misfit_gradient (precompute, workspace, forward with checkpoints, misfit, "
                     "reverse sweep with the parameter sensitivities, cell sums) and around one forward solve "
                     "(Workspace.rk4_steps, host state; precompute not included)"}
    if batch:
        # batch different seeded fields, the same observations
        fields = []
        for _ in range(batch):
            fields.append((rng.uniform(0.8, 1.25, c2.shape) ** 2, 10.0 ** rng.uniform(-6, -5, al.shape),
                           rng.uniform(0.0, 4.0, be.shape)))
        bsteps = int(round(batch_T / ((1.0 / N) / (10 * q * q))))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = W.misfit_gradients(q, N, batch_T, fields, receivers, u_obs, every=every, **kw)
        t_batch = time.perf_counter() - t0
        per_grad = t_batch / batch
        out["batch"] = {"gradients": batch, "T": batch_T, "steps": bsteps, "s": t_batch, "s_per_grad": per_grad,
                        "s_per_grad_at_T": per_grad * nsteps / bsteps,
                        "speedup_vs_single_per_step": (t_grad / nsteps) / (per_grad / bsteps),
                        "grad_over_forward_per_step": (per_grad / bsteps) / (t_fwd / nsteps),
                        "misfits": [float(r[0]) for r in res[:3]],
                        "note": "misfit_gradients: the forward runs and reverse sweeps of all gradients together, "
                                "each stage one multi-instance launch per kernel; s_per_grad_at_T scales the "
                                "per-gradient time by the steps of T"}
    return out


def main():
    global NMESH
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--mesh", type=int, default=512, help="mesh size N (profiling runs on smaller cases)")
    ap.add_argument("--state", default="front", choices=["front", "uniform", "zero"])
    ap.add_argument("--profile-only", action="store_true", help="only the main timed run (for ncu)")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-form measurement")
    ap.add_argument("--batched-only", action="store_true", help="only the batched-form measurement")
    ap.add_argument("--mass-solver", default="chebyshev", choices=["chebyshev", "cg"],
                    help="mass solver of the main workload (profiling runs of the CG kernel)")
    ap.add_argument("--general-only", action="store_true",
                    help="only the general-kernel measurement (varying coefficients; --mesh applies)")
    ap.add_argument("--adjoint", action="store_true", help="only the adjoint-form measurement (one gradient)")
    ap.add_argument("--adjoint-T", type=float, default=0.5, help="final time of the adjoint-form workload")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint-form measurement")
    ap.add_argument("--adjoint-batch", type=int, default=16, help="gradients of the adjoint-form batch")
    ap.add_argument("--adjoint-batch-T", type=float, default=0.125, help="final time of the adjoint-form batch")
    ap.add_argument("--adjoint-every", type=int, default=32, help="checkpoint interval of the adjoint form")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    NMESH = args.mesh
    KW["mass_solver"] = args.mass_solver
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
