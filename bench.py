#!/usr/bin/env python3
"""Benchmark of the Ewald mobility product on GB300.

Workload (the configuration the headline metric is quoted on): FTS mobility
product y = M x of N = 1000 equal spheres (a = 1) at volume fraction 0.30,
random-sequential-addition placement (seed 42), cubic periodic box,
x ~ N(0, 1) (seed 7), Ewald split xi = sqrt(pi)/L with libstokes' own
cutoffs for eps = 1e-12.  A step is one product over the whole system.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--precision fp64|mixed]

Prints one JSON line.  ``value`` is products per second with inputs resident
in HBM (device-timed, CUDA events on the launching stream); ``e2e`` is the
same metric through the drop-in C ABI (atimes_ewald_3all) with pinned host
buffers, host<->device copies inside the timed region.  Under torchrun each
rank runs an independent replica (the path is replicated, not sharded).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "mobility matvecs/s & BD steps/s, mixed vs FP64 on 1 GB300 at ≤1e-6 rel err"
UNIT = "matvecs/s"
WORKLOAD = dict(name="mob_fts_n1000_phi0.30", version=2, n=1000, phi=0.30, pos_seed=42,
                x_seed=7, tratio=1.0, eps=1e-12)
# reference-as-written flop count of one real-space pair term (F, FT, FTS)
FLOPS_PER_TERM = {0: 89, 1: 184, 2: 754}
L2_FLUSH_BYTES = 256 << 20


def make_inputs():
    from libstokes_gb300.workloads import forces, rsa_positions
    pos, L = rsa_positions(WORKLOAD["n"], WORKLOAD["phi"], seed=WORKLOAD["pos_seed"])
    c = (3, 6, 11)[WORKLOAD["version"]]
    x = forces(c * WORKLOAD["n"], seed=WORKLOAD["x_seed"])
    return pos, L, x


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str | None):
        self.gpu_id = gpu_id
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
               "-lms", "200"]
        if self.gpu_id is not None:
            cmd += ["-i", self.gpu_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in self.lines:
            p = [v.strip() for v in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                smax.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names[1:], p[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def gpu_pci_id(dev: int):
    try:
        import torch
        p = torch.cuda.get_device_properties(dev)
        return f"{p.pci_domain_id:08X}:{p.pci_bus_id:02X}:{p.pci_device_id:02X}.0"
    except Exception:
        return None


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (C restatement of the reference), all host cores
# ---------------------------------------------------------------------------
def cpu_baseline(pos, L, x):
    """One whole FTS product of the oracle (the C restatement of
    src/ewald.c:519-1081, OpenMP over target rows) on all host cores: its
    rate, and its output for the accuracy check of the GPU result."""
    from oracle.oracle import Oracle
    o = Oracle(WORKLOAD["version"], pos, (L, L, L))
    o.set_split(o.xi_by_tratio(WORKLOAD["tratio"]), WORKLOAD["eps"])
    threads = os.cpu_count() or 1
    o.set_threads(threads)
    t0 = time.perf_counter()
    y = o.atimes(x)
    dt = time.perf_counter() - t0
    return {"value": 1.0 / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"one whole FTS product of N = {WORKLOAD['n']} (real + reciprocal "
                      f"space, reference split), {dt:.2f} s wall on {threads} threads"}, y


def count_pairs_within(pos, L, rc):
    """Number of (i, j, lattice image) terms with 0 < r < rc in a cubic
    periodic box: the pair terms a real-space sum with cutoff rc evaluates."""
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    n = pos.shape[0]
    nsh = int(math.ceil(rc / L + 0.5))
    rng = np.arange(-nsh, nsh + 1)
    offs = np.array([(a, b, c) for a in rng for b in rng for c in rng], dtype=np.float64) * L
    rc2 = rc * rc
    total = 0
    step = max(1, 4000000 // max(n, 1))
    for i0 in range(0, n, step):
        d = pos[None, :, :] - pos[i0:i0 + step, None, :]
        d -= L * np.round(d / L)
        for o in offs:
            r2 = ((d + o) ** 2).sum(axis=-1)
            total += int(np.count_nonzero((r2 > 0.0) & (r2 < rc2)))
    return total


BD_WORKLOAD = dict(name="bd_f_n4096_phi0.20", version=0, n=4096, phi=0.20, seed=42, dt=1e-3,
                   peclet=1.0, n_cheb=30, n_lanczos=20, lj_e=1.0, lj_r0=2.0, rmin=1.0, warm=1,
                   steps=1000, steps_fp64=40, steps_dropin=4)


def _bd_engine_run(lib, abi, L, pos, Lb, precision, steps, budget_s=None):
    """Wall time of `steps` mid-point steps of the device engine (after one
    warm-up step, which also runs the Lanczos bounds); with a budget, steps
    run one at a time and stop once the budget is spent (at least one)."""
    import torch
    w = BD_WORKLOAD
    s = L.System(w["version"], pos, (Lb,) * 3)
    # real-space distances clamped at contact (libstokes' sys->rmin = 1): the
    # soft repulsion lets spheres overlap, where the unclamped far-field
    # mobility is not positive definite
    s.set_misc(rmin=w["rmin"])
    p = abi.BDParams(peclet=w["peclet"], dt=w["dt"], n_cheb=w["n_cheb"],
                     n_lanczos=w["n_lanczos"], cheb_eps=1e-2, check_every=1, lj_e=w["lj_e"],
                     lj_r0=w["lj_r0"], seed=12345, precision=precision)
    h = C.c_void_p()
    abi.check(lib.stokes_gpu_bd_create(s.sp, C.byref(p), C.byref(h)))
    abi.check(lib.stokes_gpu_bd_run(h, 0.0, w["warm"]))      # includes the Lanczos bounds
    st0 = np.zeros(4)
    abi.check(lib.stokes_gpu_bd_stats(h, st0.ctypes.data_as(abi._dp)))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if budget_s is None:
        abi.check(lib.stokes_gpu_bd_run(h, w["warm"] * w["dt"], steps))
    else:
        done = 0
        while done < steps and (done == 0 or time.perf_counter() - t0 < budget_s):
            abi.check(lib.stokes_gpu_bd_run(h, (w["warm"] + done) * w["dt"], 1))
            done += 1
        steps = done
    dt_wall = time.perf_counter() - t0
    st = np.zeros(4)
    abi.check(lib.stokes_gpu_bd_stats(h, st.ctypes.data_as(abi._dp)))
    abi.check(lib.stokes_gpu_bd_destroy(h))
    s.close()
    return {"steps_timed": steps, "steps_per_s": steps / dt_wall,
            "ms_per_step": 1000.0 * dt_wall / steps,
            "products_per_step": (st[0] - st0[0]) / steps, "cheb_err_last": st[2],
            "bound_estimates": st[1]}


def _bd_dropin_run(lib, abi, L, pos, Lb, precision, steps, budget_s=20.0):
    """Wall time per step of libstokes' own BD_evolve_mid (src/brownian.c:
    2352-2560) through this library: EV_LJ as the reference applies it
    (src/ev-LJ.c:186-265, force along the primary-cell vector), Chebyshev
    noise from BD_calc_FB with bounds estimated on the first call, host
    positions in and out every step."""
    w = BD_WORKLOAD
    n = w["n"]
    s = L.System(w["version"], pos, (Lb,) * 3)
    s.set_precision(precision)
    s.set_misc(rmin=w["rmin"])
    F = np.zeros(3 * n)
    T = np.zeros(3 * n)
    E = np.zeros(5 * n)
    lj = lib.EV_LJ_init(n)
    for i in range(n):
        lj.contents.flag[i] = 1
        lj.contents.e[i] = w["lj_e"]
        lj.contents.r0[i] = w["lj_r0"]
    dp = abi._dp
    bd = lib.BD_params_init(s.sp, 12345, F.ctypes.data_as(dp), T.ctypes.data_as(dp),
                            E.ctypes.data_as(dp), None, None, None, 0, 0, 0, 0.0, None, None,
                            1.0, None, None, None, lj, None, 0, w["peclet"], 1e-2, w["n_cheb"],
                            0, 0, 0.0, 0.0, 1e-12)
    x = np.ascontiguousarray(pos.reshape(-1).copy())
    t = 0.0
    t += lib.BD_evolve_mid(t, bd, x.ctypes.data_as(dp), None, w["dt"])   # bounds + warm-up
    t0 = time.perf_counter()
    done = 0
    while done < steps and (done == 0 or time.perf_counter() - t0 < budget_s):
        t += lib.BD_evolve_mid(t, bd, x.ctypes.data_as(dp), None, w["dt"])
        done += 1
    steps = done
    dt_wall = time.perf_counter() - t0
    abi.raise_if_failed()
    lib.BD_params_free(bd)
    lib.EV_LJ_free(lj)
    s.close()
    return {"steps_timed": steps, "steps_per_s": steps / dt_wall,
            "ms_per_step": 1000.0 * dt_wall / steps}


def bd_measure(lib, abi, L, torch, dev):
    """Brownian-dynamics steps/s: F spheres N=4096 at phi 0.20, dt 1e-3, kT 1
    (Pe 1), Chebyshev order 30 on 20-step Lanczos bounds, EV_LJ repulsion at
    r < 2 (e = 1, r0 = 2).
      * the device engine (stokes_gpu_bd_run, noise from the device generator
        in float32; EV_LJ along the nearest-image vector): all 1000 steps of
        the configuration in mixed precision, and a bounded run of the same
        engine in FP64, for the mixed / FP64 ratio;
      * libstokes' own BD_evolve_mid through this library (the reference's
        EV_LJ direction, KIrand noise, host positions): a few steps each in
        mixed and FP64 precision."""
    from libstokes_gb300.workloads import rsa_positions
    w = BD_WORKLOAD
    pos, Lb = rsa_positions(w["n"], w["phi"], seed=w["seed"])
    mixed = _bd_engine_run(lib, abi, L, pos, Lb, abi.MIXED, w["steps"])
    fp64 = _bd_engine_run(lib, abi, L, pos, Lb, abi.FP64, w["steps_fp64"], budget_s=20.0)
    d_mixed = _bd_dropin_run(lib, abi, L, pos, Lb, abi.MIXED, w["steps_dropin"])
    d_fp64 = _bd_dropin_run(lib, abi, L, pos, Lb, abi.FP64, w["steps_dropin"])
    return {"workload": w["name"], "steps_per_s": mixed["steps_per_s"],
            "ms_per_step": mixed["ms_per_step"], "steps_timed": mixed["steps_timed"],
            "products_per_step": mixed["products_per_step"],
            "cheb_err_last": mixed["cheb_err_last"], "precision": "mixed",
            "engine": {"mixed": mixed, "fp64": fp64,
                       "mixed_over_fp64": mixed["steps_per_s"] / fp64["steps_per_s"],
                       "ev_lj": "nearest-image vector (departs from src/ev-LJ.c:255-259, "
                                "which pushes along the primary-cell vector)"},
            "dropin_BD_evolve_mid": {"mixed": d_mixed, "fp64": d_fp64,
                                     "mixed_over_fp64": d_mixed["steps_per_s"]
                                     / d_fp64["steps_per_s"],
                                     "ev_lj": "as the reference (primary-cell vector)"},
            "timing": "wall clock around the runs (device engine: device-resident; drop-in: "
                      "host positions every step)",
            "params": {k: w[k] for k in ("dt", "peclet", "n_cheb", "n_lanczos", "lj_e", "lj_r0",
                                         "rmin")}}


def matrix_measure(lib, abi, L, torch, dev, pos, Lbox):
    """Dense FTS mobility matrix of the bench workload (N = 1000, 11000 x
    11000 FP64 = 968 MB) at the reference split, on device memory: device
    time (CUDA events on the builder's stream, after one warm-up build) and
    the achieved store bandwidth, against the measured HBM copy rate.  The
    FP64 builder evaluates every pair-image term of the reference split in
    FP64, so the FP64 pipe bounds it.  The split-precision builder
    (k_matrix_pairs: FP32 terms at its own split, each unordered pair once,
    both blocks stored) is bound by its FP32 issue rate."""
    w = WORKLOAD
    s = L.System(w["version"], pos, (Lbox,) * 3, tratio=w["tratio"], eps=w["eps"])
    n = (3, 6, 11)[w["version"]] * w["n"]
    d_pos = torch.tensor(pos, dtype=torch.float64, device=dev).contiguous()
    d_mat = torch.empty((n, n), dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream(dev)
    sp = C.c_void_p(st.cuda_stream)
    abi.check(lib.stokes_gpu_matrix_dev(s.sp, C.c_void_p(d_pos.data_ptr()),
                                        C.c_void_p(d_mat.data_ptr()), sp))
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    abi.check(lib.stokes_gpu_matrix_dev(s.sp, C.c_void_p(d_pos.data_ptr()),
                                        C.c_void_p(d_mat.data_ptr()), sp))
    e1.record(st)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1)
    nbytes = 8.0 * n * n
    peak = measured_peaks().get("hbm_gbs")
    P = C.c_longlong()
    abi.check(lib.stokes_gpu_count_real_terms_dense(s.sp, C.byref(P)))
    # the split-precision builder (FP32 terms, FP64 entries) on the same
    # system, and its largest entry error against the FP64 matrix
    s.set_precision(abi.MIXED)
    d_m32 = torch.empty_like(d_mat)
    abi.check(lib.stokes_gpu_matrix_dev(s.sp, C.c_void_p(d_pos.data_ptr()),
                                        C.c_void_p(d_m32.data_ptr()), sp))
    torch.cuda.synchronize(dev)
    e0.record(st)
    abi.check(lib.stokes_gpu_matrix_dev(s.sp, C.c_void_p(d_pos.data_ptr()),
                                        C.c_void_p(d_m32.data_ptr()), sp))
    e1.record(st)
    torch.cuda.synchronize(dev)
    ms32 = e0.elapsed_time(e1)
    err32 = float((d_m32 - d_mat).abs().max() / d_mat.abs().max())
    s.close()
    del d_mat, d_m32
    torch.cuda.empty_cache()
    gbs = nbytes / (ms * 1e-3) / 1e9
    return {"workload": f"matrix_fts_n{w['n']}_phi{w['phi']:.2f}", "precision": "fp64",
            "ms": ms, "bytes": nbytes, "achieved_gbs": gbs, "hbm_peak_gbs": peak,
            "hbm_frac": gbs / peak if peak else None,
            "pair_image_terms": P.value, "terms_per_s": P.value / (ms * 1e-3),
            "mixed": {"ms": ms32, "achieved_gbs": nbytes / (ms32 * 1e-3) / 1e9,
                      "hbm_frac": (nbytes / (ms32 * 1e-3) / 1e9) / peak if peak else None,
                      "max_err_over_max_entry": err32,
                      "precision": "FP32 terms, FP64 entries (k_matrix_pairs)"},
            "bound": "fp64-pipe: every pair-image term of the reference split "
                     "(xi = sqrt(pi)/L, eps 1e-12) builds an 11 x 11 block in FP64"}


def lub_measure(lib, abi, L, torch, dev, reps: int = 20):
    """Lubrication correction (calc_lub_3ft, src/lub.c:370) of FT, N = 1000,
    phi 0.35 (rsa seed 71), lubmax 3, lubmin2 2.0001^2, FP64 on device
    buffers: device time per application (CUDA events over `reps` after
    three warm-ups), the close pairs it visits, and one lubricated mobility
    solve (I + M L) u = M f (STOKES_GPU_SOLVE_MOB_LUB, mixed product with
    FP64 refinement) against the CPU oracle's time for one application on
    all host threads."""
    from libstokes_gb300.workloads import rsa_positions
    from oracle.oracle import calc_lub
    n = 1000
    pos, Lb = rsa_positions(n, 0.35, seed=71)
    s = L.System(1, pos, (Lb,) * 3)
    s.s.lubmin2 = 2.0001 ** 2
    s.s.lubmax = 3.0
    u = np.random.default_rng(72).standard_normal(6 * n)
    d_pos = torch.tensor(pos, dtype=torch.float64, device=dev).contiguous()
    d_u = torch.tensor(u, dtype=torch.float64, device=dev)
    d_f = torch.empty_like(d_u)
    st = torch.cuda.current_stream(dev)
    sp = C.c_void_p(st.cuda_stream)

    def apply():
        abi.check(lib.stokes_gpu_lub_dev(s.sp, 1, C.c_void_p(d_pos.data_ptr()),
                                         C.c_void_p(d_u.data_ptr()), C.c_void_p(d_f.data_ptr()),
                                         sp))
    for _ in range(3):
        apply()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        apply()
    e1.record(st)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / reps
    f = d_f.cpu().numpy()
    d = pos[None, :, :] - pos[:, None, :]
    d -= Lb * np.rint(d / Lb)
    r2 = (d ** 2).sum(-1)
    close = int(((r2 > 0) & (r2 < 9.0)).sum())
    t0 = time.perf_counter()
    fo = calc_lub(1, pos, (Lb,) * 3, u, lubmin2=2.0001 ** 2, lubmax=3.0)
    cpu_s = time.perf_counter() - t0
    err = float(np.linalg.norm(f - fo) / np.linalg.norm(fo))
    # the lubricated mobility problem with the mixed product
    s.set_precision(abi.MIXED)
    b = s.atimes(np.random.default_rng(73).standard_normal(6 * n))
    x = np.zeros(6 * n)
    it, res = C.c_int(), C.c_double()
    t0 = time.perf_counter()
    abi.check(lib.stokes_gpu_solve(s.sp, abi.SOLVE_MOB_LUB, b.ctypes.data_as(abi._dp),
                                   x.ctypes.data_as(abi._dp), 30, 2000, 1e-10, C.byref(it),
                                   C.byref(res)))
    solve_s = time.perf_counter() - t0
    s.close()
    return {"workload": "lub_ft_n1000_phi0.35_lubmax3", "precision": "fp64",
            "ms_per_application": ms, "applications_per_s": 1000.0 / ms,
            "close_pairs_ordered": close, "rel_err_vs_oracle": err,
            "solve_mob_lub": {"wall_s": solve_s, "applications": it.value, "residual": res.value,
                              "precision": "mixed product, FP64 refinement"},
            "cpu_baseline": {"applications_per_s": 1.0 / cpu_s, "cores": 1, "kind": "port",
                             "sample": "one application of the oracle (oracle_calc_lub, serial)"}}


def open_measure(lib, abi, L, torch, dev, pos, reps: int = 20):
    """Free-space FTS product (atimes_nonewald_3all, src/non-ewald.c:330-481)
    of the bench's N = 1000 spheres as an open system, FP64, device buffers:
    device time per product (CUDA events over `reps` products after three
    warm-up products) and the pair rate, beside the CPU oracle's time for one
    product on all host threads."""
    from oracle.oracle import Oracle
    w = WORKLOAD
    s = L.System(2, pos, periodic=False)
    n = 11 * w["n"]
    rng = np.random.default_rng(5)
    x = rng.standard_normal(n)
    d_pos = torch.tensor(pos, dtype=torch.float64, device=dev).contiguous()
    d_x = torch.tensor(x, dtype=torch.float64, device=dev)
    d_y = torch.empty_like(d_x)
    st = torch.cuda.current_stream(dev)
    sp = C.c_void_p(st.cuda_stream)

    def product():
        abi.check(lib.stokes_gpu_atimes_dev(s.sp, C.c_void_p(d_pos.data_ptr()),
                                            C.c_void_p(d_x.data_ptr()),
                                            C.c_void_p(d_y.data_ptr()), sp))
    def timed():
        for _ in range(3):
            product()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            product()
        e1.record(st)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / reps
    ms = timed()
    y64 = d_y.cpu().numpy()
    s.set_precision(abi.MIXED)
    ms_mixed = timed()
    err_mixed = float(np.linalg.norm(d_y.cpu().numpy() - y64) / np.linalg.norm(y64))
    s.close()
    o = Oracle(2, pos, (1.0, 1.0, 1.0))
    threads = os.cpu_count() or 1
    o.set_threads(threads)
    t0 = time.perf_counter()
    o.atimes_nonewald(x)
    cpu_s = time.perf_counter() - t0
    pairs = w["n"] * (w["n"] - 1)
    return {"workload": f"open_fts_n{w['n']}", "precision": "fp64", "ms_per_product": ms,
            "products_per_s": 1000.0 / ms, "pairs_per_s": pairs / (ms * 1e-3),
            "mixed": {"ms_per_product": ms_mixed, "products_per_s": 1000.0 / ms_mixed,
                      "pairs_per_s": pairs / (ms_mixed * 1e-3), "rel_err_vs_fp64": err_mixed},
            "cpu_baseline": {"products_per_s": 1.0 / cpu_s, "cores": threads, "kind": "port",
                             "sample": "one full product of the oracle (oracle_atimes_nonewald)"},
            "bound": "fp64-pipe: N(N-1) ordered pairs, each the free-space scalars and "
                     "the 11 x 11 pair tensor applied in FP64"}


def solve_measure(lib, abi, L, torch, dev, pos, Lbox, product_ms, eps=1e-10):
    """FTS resistance solve M x = b (solve_iter with atimes_3all, the call of
    src/ewald-3fts.c:71) on the bench's N = 1000 spheres to eps 1e-10 from a
    zero start: mixed precision (GMRES(30) on the mixed product inside FP64
    iterative refinement; every residual test uses the FP64 product) against
    the plain FP64 GMRES(30) solve; wall time of the whole solve (host
    buffers in and out), operator applications, and the relative difference
    of the two solutions."""
    w = WORKLOAD
    s = L.System(w["version"], pos, (Lbox,) * 3, tratio=w["tratio"], eps=w["eps"])
    n = s.n
    b = np.random.default_rng(11).standard_normal(n)
    it = C.c_int()
    res = C.c_double()
    out = {"workload": f"solve_res_fts_n{w['n']}_phi{w['phi']:.2f}", "eps": eps}
    sols = {}
    for name, prec, reps in (("mixed_refined", abi.MIXED, 3), ("fp64", abi.FP64, 1)):
        s.set_precision(prec)
        x = np.zeros(n)
        abi.check(lib.stokes_gpu_solve(s.sp, 0, abi._d(b), abi._d(x), 30, 5000, 1e-4,
                                       C.byref(it), C.byref(res)))  # warm-up: graphs, workspace
        walls = []
        for _ in range(reps):
            x[:] = 0.0
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            abi.check(lib.stokes_gpu_solve(s.sp, 0, abi._d(b), abi._d(x), 30, 5000, eps,
                                           C.byref(it), C.byref(res)))
            walls.append(time.perf_counter() - t0)
        sols[name] = x.copy()
        out[name] = {"ms": 1000.0 * float(np.median(walls)), "applications": it.value,
                     "relative_residual_fp64": res.value,
                     "ms_runs": [1000.0 * t for t in walls]}
    s.close()
    out["mixed_refined"]["solver"] = ("GMRES(30) on the mixed product inside FP64 iterative "
                                      "refinement (residuals from the FP64 product)")
    out["fp64"]["solver"] = "GMRES(30) on the FP64 product"
    out["speedup_mixed_refined_over_fp64"] = out["fp64"]["ms"] / out["mixed_refined"]["ms"]
    out["rel_diff_solutions"] = float(np.linalg.norm(sols["mixed_refined"] - sols["fp64"])
                                      / np.linalg.norm(sols["fp64"]))
    out["product_ms_mixed"] = product_ms
    out["timing"] = "wall clock around stokes_gpu_solve (host buffers), median of 3 (mixed), 1 (fp64)"
    return out


def scale_measure(lib, abi, L, torch, dev, sizes=(4096, 16384), reps=10):
    """The mixed FTS product at larger N (phi 0.30, the same placement
    rule): products/s on device buffers (CUDA events on a side stream), the
    per-kernel times of a separate profiled pass, and the roofline of the
    dominant main-stream kernel, to show how the kernels behave as the
    tensor-core GEMMs grow past the bench workload's small tiles."""
    from libstokes_gb300.workloads import rsa_positions
    out = []
    for n in sizes:
        pos, Lb = rsa_positions(n, WORKLOAD["phi"], seed=WORKLOAD["pos_seed"])
        s = L.System(2, pos, (Lb,) * 3, tratio=WORKLOAD["tratio"], eps=WORKLOAD["eps"])
        s.set_precision(abi.MIXED)
        d_pos = torch.tensor(pos, dtype=torch.float64, device=dev).contiguous()
        d_x = torch.randn(11 * n, dtype=torch.float64, device=dev)
        d_y = torch.empty_like(d_x)
        st = torch.cuda.Stream(dev)
        sp = C.c_void_p(st.cuda_stream)

        def product():
            abi.check(lib.stokes_gpu_atimes_dev(s.sp, C.c_void_p(d_pos.data_ptr()),
                                                C.c_void_p(d_x.data_ptr()),
                                                C.c_void_p(d_y.data_ptr()), sp))
        with torch.cuda.stream(st):
            for _ in range(3):
                product()
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for _ in range(reps):
                product()
            e1.record(st)
            torch.cuda.synchronize(dev)
            ms = e0.elapsed_time(e1) / reps
            abi.check(lib.stokes_gpu_kprof_begin(s.sp, 16 * 3))
            for _ in range(3):
                product()
            torch.cuda.synchronize(dev)
        kprof = abi.kernel_profile(lib, s.sp)
        kernels_ms = {k: v[0] / max(v[1], 1) for k, v in kprof.items()}
        wl = f"mob_fts_n{n}_phi{WORKLOAD['phi']:.2f}"
        roof = roofline(lib, abi, s, 2, n, 11, kernels_ms, "mixed", workload=wl)
        # accuracy of the timed output against the FP64 path on the same inputs
        y_mixed = d_y.cpu().numpy()
        s.set_precision(abi.FP64)
        with torch.cuda.stream(st):
            product()
            torch.cuda.synchronize(dev)
        y64 = d_y.cpu().numpy()
        err = float(np.linalg.norm(y_mixed - y64) / np.linalg.norm(y64))
        s.close()
        out.append({"n": n, "workload": wl, "ms_per_product": ms, "products_per_s": 1000.0 / ms,
                    "rel_err_vs_fp64": err, "kernels_ms": kernels_ms,
                    "roofline": {k: roof.get(k) for k in ("kernel", "achieved", "peak", "frac",
                                                          "kernel_ms", "unit", "main_stream")}})
    return out


ADJ_WORKLOAD = dict(name="vjp_ft_n2048_phi0.25", version=1, n=2048, phi=0.25, seed=42)


def adjoint_measure(lib, abi, L):
    """Vector-Jacobian product of L = g . M(r) f (FT, N = 2048, phi 0.25,
    g, f ~ N(0,1)) against one forward product on the same system, both
    FP64 through the host API (wall clock, copies included)."""
    from libstokes_gb300.workloads import rsa_positions
    w = ADJ_WORKLOAD
    pos, Lb = rsa_positions(w["n"], w["phi"], seed=w["seed"])
    s = L.System(w["version"], pos, (Lb,) * 3)
    c = (3, 6, 11)[w["version"]]
    rng = np.random.default_rng(1)
    g = rng.standard_normal(c * w["n"])
    f = rng.standard_normal(c * w["n"])
    dr = np.zeros(3 * w["n"])
    db = np.zeros(3)
    Lv = C.c_double()
    dp = abi._dp

    def vjp():
        abi.check(lib.stokes_gpu_vjp(s.sp, g.ctypes.data_as(dp), f.ctypes.data_as(dp),
                                     dr.ctypes.data_as(dp), db.ctypes.data_as(dp), None))

    s.atimes(f)
    vjp()
    t0 = time.perf_counter()
    s.atimes(f)
    fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    vjp()
    adj = time.perf_counter() - t0
    dr64, db64 = dr.copy(), db.copy()
    # mixed precision: the FP32 adjoint against the mixed forward product
    s.set_precision(abi.MIXED)
    for _ in range(3):
        s.atimes(f)
        vjp()
    fw, aw = [], []
    for _ in range(5):
        t0 = time.perf_counter()
        s.atimes(f)
        fw.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        vjp()
        aw.append(time.perf_counter() - t0)
    fwd_m, adj_m = float(np.median(fw)), float(np.median(aw))
    err_r = float(np.linalg.norm(dr - dr64) / np.linalg.norm(dr64))
    err_b = float(np.abs(db - db64).max() / np.abs(db64).max())
    s.close()
    return {"workload": w["name"], "precision": "fp64", "forward_s": fwd, "vjp_s": adj,
            "vjp_over_forward": adj / fwd, "outputs": "dL/dr (6144) and dL/dl (3)",
            "mixed": {"forward_s": fwd_m, "vjp_s": adj_m, "vjp_over_forward": adj_m / fwd_m,
                      "rel_err_dLdr_vs_fp64": err_r, "rel_err_dLdbox_vs_fp64": err_b,
                      "timing": "median of 5 calls each, host buffers"},
            "timing": "wall clock around one call each, host buffers"}


def fit_measure(lib, abi, L, steps=200):
    """Positions fitted to a target velocity field (FT, N = 2048, phi 0.25):
    loss |M(r) f - u*|^2 with u* = M(r*) f at r* = r + 0.05 N(0,1), the
    gradient from the VJP at g = 2 (M f - u*), a step along -gradient with
    backtracking (halve until the loss falls, then double the next trial).
    Every step runs one VJP and one or more FP64 forward products through
    the host API."""
    from libstokes_gb300.workloads import rsa_positions
    w = ADJ_WORKLOAD
    pos, Lb = rsa_positions(w["n"], w["phi"], seed=w["seed"])
    c = (3, 6, 11)[w["version"]]
    rng = np.random.default_rng(10)
    f = rng.standard_normal(c * w["n"])
    t = L.System(w["version"], pos + 0.05 * rng.standard_normal(pos.shape), (Lb,) * 3)
    u_star = t.atimes(f)
    t.close()
    s = L.System(w["version"], pos, (Lb,) * 3)
    dp = abi._dp
    dr = np.zeros(3 * w["n"])
    db = np.zeros(3)

    def loss_at(x):
        lib.stokes_set_pos(s.sp, x.ctypes.data_as(dp))
        r = s.atimes(f) - u_star
        return float(r @ r), r

    x = pos.reshape(-1).copy()
    lv, r = loss_at(x)
    l0 = lv
    step, products = 1e-3, 1
    t0 = time.perf_counter()
    for _ in range(steps):
        g = 2.0 * r
        abi.check(lib.stokes_gpu_vjp(s.sp, g.ctypes.data_as(dp), f.ctypes.data_as(dp),
                                     dr.ctypes.data_as(dp), db.ctypes.data_as(dp), None))
        for _ in range(30):
            xn = x - step * dr
            ln, rn = loss_at(xn)
            products += 1
            if ln < lv:
                break
            step *= 0.5
        if not ln < lv:
            break
        x, lv, r = xn, ln, rn
        step *= 2.0
    wall = time.perf_counter() - t0
    s.close()
    return {"workload": "fit_ft_n2048_phi0.25_200steps", "steps": steps, "wall_s": wall,
            "s_per_step": wall / steps, "forward_products": products, "loss_initial": l0,
            "loss_final": lv, "loss_ratio": lv / l0, "precision": "fp64 forward and VJP",
            "timing": "wall clock, host buffers"}


BATCH_WORKLOAD = dict(name="ensemble_512_n16-512_phi0.05-0.35_F_FT", nsys=512, nmin=16,
                      nmax=512, phimin=0.05, phimax=0.35, seed=2024, bd_steps=10, n_cheb=30)


def batch_measure(lib, abi, L, nsys=None):
    """Ensemble of independent periodic systems (N ~ U{16..512}, phi ~
    U[0.05, 0.35], F and FT alternating, forces N(0,1) float32): one batched
    mixed product of all systems and 10 batched BD steps (Chebyshev 30 on
    20-step Lanczos bounds, device noise), against a host loop of
    single-system mixed products over the first 32 systems."""
    from libstokes_gb300.workloads import rsa_positions
    w = BATCH_WORKLOAD
    ns = nsys or w["nsys"]
    rng = np.random.default_rng(w["seed"])
    systems = []
    for s in range(ns):
        n = int(rng.integers(w["nmin"], w["nmax"] + 1))
        phi = float(rng.uniform(w["phimin"], w["phimax"]))
        pos, Lb = rsa_positions(n, phi, seed=w["seed"] + s)
        systems.append(L.System(s % 2, pos, (Lb,) * 3))
    arr = (C.POINTER(abi.StokesStruct) * ns)(*[sy.sp for sy in systems])
    h = C.c_void_p()
    t0 = time.perf_counter()
    abi.check(lib.stokes_gpu_batch_create(arr, ns, abi.MIXED, C.byref(h)))
    t_create = time.perf_counter() - t0
    npt, nt = C.c_int(), C.c_int()
    lib.stokes_gpu_batch_size(h, C.byref(npt), C.byref(nt))
    x = rng.standard_normal(nt.value).astype(np.float32).astype(np.float64)
    y = np.zeros(nt.value)
    dp = abi._dp
    t0 = time.perf_counter()
    abi.check(lib.stokes_gpu_batch_atimes(h, x.ctypes.data_as(dp), y.ctypes.data_as(dp)))
    t_tune = time.perf_counter() - t0
    reps, dev_ms = 5, []
    st = np.zeros(4)
    t0 = time.perf_counter()
    for _ in range(reps):
        abi.check(lib.stokes_gpu_batch_atimes(h, x.ctypes.data_as(dp), y.ctypes.data_as(dp)))
        lib.stokes_gpu_batch_stats(h, st.ctypes.data_as(dp))
        dev_ms.append(st[0])
    t_prod = (time.perf_counter() - t0) / reps
    etas = []
    for s in range(ns):
        eta = C.c_double()
        abi.check(lib.stokes_gpu_batch_split(h, s, C.byref(eta), None))
        etas.append(eta.value)
    t0 = time.perf_counter()
    abi.check(lib.stokes_gpu_batch_bd(h, 1.0, 1e-3, w["n_cheb"], 20, None, None, 11,
                                      w["bd_steps"], None))
    t_bd = time.perf_counter() - t0
    abi.check(lib.stokes_gpu_batch_destroy(h))
    # the per-system alternative: a host loop of single-system products
    loop = systems[:32]
    xs = [rng.standard_normal(sy.n) for sy in loop]
    for sy, xv in zip(loop, xs):
        sy.set_precision(abi.MIXED)
        sy.atimes(xv)
    t0 = time.perf_counter()
    for sy, xv in zip(loop, xs):
        sy.atimes(xv)
    t_loop = (time.perf_counter() - t0) / len(loop) * ns
    for sy in systems:
        sy.close()
    return {"workload": w["name"], "systems": ns, "particles": npt.value, "precision": "mixed",
            "batch_product_ms_device": float(np.median(dev_ms)),
            "batch_product_ms_wall": 1000.0 * t_prod,
            "system_products_per_s": ns / t_prod,
            "bd_steps": w["bd_steps"], "bd_wall_s": t_bd,
            "systems_per_s_product_plus_bd": ns / (t_prod + t_bd),
            "host_loop_product_ms_extrapolated": 1000.0 * t_loop,
            "batch_over_host_loop": t_loop / t_prod,
            "autotuned": {"chunk_mult": st[1], "real_warps_per_cta": st[2],
                          "eta_min": min(etas), "eta_max": max(etas)},
            "create_s": t_create, "first_product_with_autotune_s": t_tune,
            "k_vectors_total": st[3]}


def run_reference(args):
    """--impl reference: the reference's CPU algorithm (the oracle port; the
    reference sources themselves are not on this machine) on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    pos, L, x = make_inputs()
    from oracle.oracle import Oracle
    o = Oracle(WORKLOAD["version"], pos, (L, L, L))
    o.set_split(o.xi_by_tratio(WORKLOAD["tratio"]), WORKLOAD["eps"])
    threads = os.cpu_count() or 1
    o.set_threads(threads)
    n = WORKLOAD["n"]
    times = []
    t_all = time.perf_counter()
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        o.atimes(x)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
    t_all = time.perf_counter() - t_all
    ms = 1000.0 * sum(times) / len(times)
    value = 1000.0 / ms
    xi_ref = o.xi_by_tratio(WORKLOAD["tratio"])
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD["name"], "version": "FTS", "n_particles": n,
                       "phi": WORKLOAD["phi"], "box": L, "xi": xi_ref,
                       "ewald_eps": WORKLOAD["eps"], "precision": "fp64"},
            "wall_s_all_steps": t_all,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"each step: one whole FTS product of N = {n} (all "
                                       "target rows, real + reciprocal space)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    return json.load(open(path)) if os.path.exists(path) else {}


def roofline(lib, abi, sysm, version, n, c, kernels_ms, precision, workload=None) -> dict:
    """Roofline of the dominant kernel of one product: algorithmic flops of
    that kernel per launch over its CUDA-event time (events on the stream it
    is launched on, in the profiling pass, where every kernel runs alone in
    order), against the peak of the pipe that bounds it.  Dominant: the
    longest kernel.  In the timed products the mixed real-space sum
    (mk_real) runs on a low-priority side stream beside the reciprocal
    chain; the longest kernel of the product's own stream is reported as
    `main_stream`."""
    side = {"mk_real"}
    name = max(kernels_ms, key=kernels_ms.get)
    out = roofline_of(lib, abi, sysm, version, n, c, kernels_ms, precision, name, workload)
    main = {k: v for k, v in kernels_ms.items() if k not in side}
    if main:
        mname = max(main, key=main.get)
        if mname != name:
            sec = roofline_of(lib, abi, sysm, version, n, c, kernels_ms, precision, mname,
                              workload)
            out["main_stream"] = {k: sec.get(k) for k in ("kernel", "bound", "achieved", "peak",
                                                          "unit", "frac", "traffic",
                                                          "kernel_ms", "algorithmic")}
    return out


def roofline_of(lib, abi, sysm, version, n, c, kernels_ms, precision, name, workload=None):
    ms = kernels_ms[name]
    peaks = measured_peaks()
    if name in ("k_sfac_gemm", "k_bp_gemm", "mk_sfac", "mk_backproj"):
        # reciprocal space: the forward sum or the back-projection, 4 Nk N c
        # flops each (Nk: the full k sphere of the split)
        info = np.zeros(9)
        abi.check(lib.stokes_gpu_mixed_split(sysm.sp, info.ctypes.data_as(abi._dp)))
        nk_full = 2 * int(info[5])
        units = nk_full * n * c
        algo = {"unit": "k vector x particle x component (full k sphere)",
                "units_per_launch": units, "flops_per_unit": 4, "k_vectors": nk_full,
                "mixed_split": {"xi": info[0], "rc": info[1], "kc": info[2], "eta": info[3],
                                "eps": info[4]}}
        flops = 4.0 * units
        if name.startswith("k_"):
            bound = "tensor"
            peak = peaks.get("bf16_tflops", 1900.0) / 2.0
            psrc = ("TF32 dense rate taken as half the measured bf16 GEMM rate "
                    "(MEASURED_PEAKS.json bf16_tflops / 2); the 3xTF32 split executes 3x "
                    "the algorithmic count and the m1 >= 0 box about 2x more")
        else:
            bound = "fp32-pipe"
            pk = C.c_double()
            abi.check(lib.stokes_gpu_peak_fma(0, C.byref(pk)))
            peak = pk.value / 1e3
            psrc = "FP32 FMA rate measured in this run by an FMA-chain kernel"
    elif name == "mk_real":
        # FP32 real space of the mixed split: every (i, j, image) term the
        # kernel evaluates, counted on the device with the kernel's own test
        P = C.c_longlong()
        abi.check(lib.stokes_gpu_count_mixed_real_terms(sysm.sp, C.byref(P)))
        info = np.zeros(9)
        abi.check(lib.stokes_gpu_mixed_split(sysm.sp, info.ctypes.data_as(abi._dp)))
        flops = float(P.value) * FLOPS_PER_TERM[version]
        algo = {"unit": "pair-image interaction (mixed split)", "units_per_launch": P.value,
                "flops_per_unit": FLOPS_PER_TERM[version],
                "mixed_split": {"xi": info[0], "rc": info[1], "kc": info[2], "eta": info[3],
                                "eps": info[4]}}
        bound = "fp32-pipe"
        pk = C.c_double()
        abi.check(lib.stokes_gpu_peak_fma(0, C.byref(pk)))
        peak = pk.value / 1e3
        psrc = "FP32 FMA rate measured in this run by an FMA-chain kernel"
    elif name == "k_real":
        P = C.c_longlong()
        abi.check(lib.stokes_gpu_count_real_terms(sysm.sp, C.byref(P)))
        flops = float(P.value) * FLOPS_PER_TERM[version]
        algo = {"unit": "pair-image interaction", "units_per_launch": P.value,
                "flops_per_unit": FLOPS_PER_TERM[version]}
        bound = "fp64-pipe"
        pk = C.c_double()
        abi.check(lib.stokes_gpu_peak_fma(1, C.byref(pk)))
        peak = pk.value / 1e3
        psrc = "FP64 FMA rate measured in this run by an FMA-chain kernel"
    else:
        return {"kernel": name, "kernel_ms": ms, "achieved": None, "peak": None,
                "frac": None, "traffic": None, "note": "no algorithmic count for this kernel"}
    achieved = flops / (ms * 1e-3) / 1e12
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        traffic = json.load(open(tpath)).get(f"{workload or WORKLOAD['name']}:{precision}:{name}")
    return {"kernel": name, "bound": bound, "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
            "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + write.sum)",
            "kernel_ms": ms, "algorithmic": algo, "peak_source": psrc}


def max_over_ranks(v: float, world: int, dev=None) -> float:
    """The largest value over the ranks of the initialised process group (the
    slowest replica sets the step time); the value itself for one rank."""
    if world <= 1:
        return float(v)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(ms_max: float, world: int) -> float:
    """Whole-job products/s: every replica does one product per step, the
    step lasting as long as the slowest replica's."""
    return world * 1000.0 / ms_max


def run_gpu(args):
    import torch
    import libstokes_gb300 as L
    from libstokes_gb300 import abi

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    lib = L.load()
    pos, Lbox, x = make_inputs()
    version, n = WORKLOAD["version"], WORKLOAD["n"]
    sysm = L.System(version, pos, (Lbox,) * 3, tratio=WORKLOAD["tratio"], eps=WORKLOAD["eps"])
    prec = abi.MIXED if args.precision == "mixed" else abi.FP64
    sysm.set_precision(prec)

    d_pos = torch.tensor(pos, dtype=torch.float64, device=dev).contiguous()
    d_x = torch.tensor(x, dtype=torch.float64, device=dev)
    d_y = torch.empty_like(d_x)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    # a dedicated stream: the library's kernels, the flush and the timing
    # events all go to it (the legacy default stream would not order them)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sp = C.c_void_p(stream.cuda_stream)

    def product():
        abi.check(lib.stokes_gpu_atimes_dev(sysm.sp, C.c_void_p(d_pos.data_ptr()),
                                            C.c_void_p(d_x.data_ptr()),
                                            C.c_void_p(d_y.data_ptr()), sp))

    for _ in range(args.warmup):
        product()
    torch.cuda.synchronize(dev)

    # accuracy of this precision against the FP64 path on the same inputs
    y_this = d_y.double().cpu().numpy()
    if prec != abi.FP64:
        ref = L.System(version, pos, (Lbox,) * 3, tratio=WORKLOAD["tratio"], eps=WORKLOAD["eps"])
        y64 = ref.atimes(x)
        ref.close()
    else:
        y64 = y_this
    rel_err = float(np.linalg.norm(y_this - y64) / np.linalg.norm(y64))

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(gpu_pci_id(local)) as clk:
        t_wall0 = time.perf_counter()
        for k in range(args.steps):
            flush.fill_(k & 0xFF)            # evict L2 between steps (not timed)
            starts[k].record(stream)
            product()
            ends[k].record(stream)
        torch.cuda.synchronize(dev)
        t_wall = time.perf_counter() - t_wall0
        barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    # the output of the last timed product, for the accuracy check against
    # the oracle's FP64 product of the same inputs
    y_timed = d_y.double().cpu().numpy()
    # per-kernel and per-phase device times: a separate, untimed pass (the
    # profiling windows record an event after every kernel)
    abi.check(lib.stokes_gpu_profile_begin(sysm.sp, args.steps))
    abi.check(lib.stokes_gpu_kprof_begin(sysm.sp, 16 * args.steps))
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        product()
    torch.cuda.synchronize(dev)
    kprof = abi.kernel_profile(lib, sysm.sp)
    prof = np.zeros(3)
    cnt = C.c_int()
    abi.check(lib.stokes_gpu_profile_end(sysm.sp, prof.ctypes.data_as(C.POINTER(C.c_double)),
                                         C.byref(cnt)))
    ms = max_over_ranks(sum(step_ms) / len(step_ms), world, dev)
    value = aggregate_rate(ms, world)
    launches = C.c_int()
    abi.check(lib.stokes_gpu_last_launches(sysm.sp, C.byref(launches)))

    # end to end through the drop-in ABI with pinned host buffers
    hx = torch.from_numpy(x).pin_memory()
    hy = torch.empty(x.size, dtype=torch.float64).pin_memory()
    px = C.cast(C.c_void_p(hx.data_ptr()), abi._dp)
    py = C.cast(C.c_void_p(hy.data_ptr()), abi._dp)
    nvec = x.size
    for _ in range(max(1, args.warmup)):
        lib.atimes_ewald_3all(nvec, px, py, C.cast(sysm.sp, C.c_void_p))
    barrier()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        lib.atimes_ewald_3all(nvec, px, py, C.cast(sysm.sp, C.c_void_p))
    torch.cuda.synchronize(dev)
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, world, dev)
    abi.raise_if_failed()
    # the same through plain (pageable, malloc'd) host arrays, as a libstokes
    # caller passes them: the library stages them through its own buffers
    px_pg = np.ascontiguousarray(x.copy())
    py_pg = np.empty_like(px_pg)
    ppx, ppy = px_pg.ctypes.data_as(abi._dp), py_pg.ctypes.data_as(abi._dp)
    for _ in range(max(1, args.warmup)):
        lib.atimes_ewald_3all(nvec, ppx, ppy, C.cast(sysm.sp, C.c_void_p))
    barrier()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        lib.atimes_ewald_3all(nvec, ppx, ppy, C.cast(sysm.sp, C.c_void_p))
    torch.cuda.synchronize(dev)
    e2e_pg_s = max_over_ranks((time.perf_counter() - t0) / args.steps, world, dev)
    abi.raise_if_failed()

    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    c = (3, 6, 11)[version]
    real_ms = prof[1] / max(cnt.value, 1)
    recip_ms = prof[2] / max(cnt.value, 1)
    total_ms = prof[0] / max(cnt.value, 1)
    fp64 = prec == abi.FP64
    kernels_ms = {k: v[0] / max(v[1], 1) for k, v in kprof.items()}
    roof = roofline(lib, abi, sysm, version, n, c, kernels_ms, args.precision)
    split = {}
    if not fp64:
        info = np.zeros(9)
        abi.check(lib.stokes_gpu_mixed_split(sysm.sp, info.ctypes.data_as(abi._dp)))
        split = {"mixed_split": {"xi": info[0], "eta": info[3], "rc": info[1], "kc": info[2],
                                 "eps": info[4], "k_vectors_half_space": int(info[5])}}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if fp64 else "f32 (self term and final sum f64)",
        "data": "synthetic (seeded RSA placement, N(0,1) forces)",
        "config": {"workload": WORKLOAD["name"], "version": "FTS", "n_particles": n,
                   "phi": WORKLOAD["phi"], "box": Lbox,
                   "xi": (split["mixed_split"]["xi"] if split else sysm.s.xi),
                   "ewald_eps": (split["mixed_split"]["eps"] if split else WORKLOAD["eps"]),
                   "reference_split": {"xi": sysm.s.xi, "eps": WORKLOAD["eps"],
                                       "n_images": sysm.s.nr,
                                       "note": "libstokes' own split (xi = sqrt(pi)/L), set "
                                               "on the struct; the accuracy reference"},
                   **split, "precision": args.precision,
                   "l2": "flushed between steps by a 256 MiB write outside the per-step events",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "rel_err_vs_fp64": rel_err,
        "phases_ms": {"total": total_ms, "real": real_ms, "reciprocal": recip_ms},
        "kernels_ms": kernels_ms,
        "wall_s_timed_region": t_wall,
        "gpu_launches": launches.value * args.steps,
        "e2e": {"value": world / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": 8 * (3 * n + c * n),
                "d2h_bytes_per_step": 8 * c * n,
                "path": "atimes_ewald_3all (src/ewald.h:155-156) with pinned host x and y"},
        "e2e_pageable": {"value": world / e2e_pg_s, "unit": UNIT,
                         "h2d_bytes_per_step": 8 * (3 * n + c * n),
                         "d2h_bytes_per_step": 8 * c * n,
                         "path": "atimes_ewald_3all with plain pageable numpy arrays"},
        "roofline": roof,
        "clocks": clk.summary(),
    }
    if not fp64 and not args.no_fp64_compare:
        # the plain FP64 path on the same inputs, for the mixed/FP64 ratio
        sysm.set_precision(abi.FP64)
        for _ in range(1):
            product()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            product()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        fp64_ms = e0.elapsed_time(e1) / 3
        line["fp64_path"] = {"value": 1000.0 / fp64_ms, "unit": UNIT, "ms_per_step": fp64_ms,
                             "mixed_over_fp64": (1000.0 / ms) / (1000.0 / fp64_ms)}
    if not args.no_matrix:
        line["matrix"] = matrix_measure(lib, abi, L, torch, dev, pos, Lbox)
    if not args.no_open:
        line["open"] = open_measure(lib, abi, L, torch, dev, pos)
    if not args.no_solve and not fp64:
        line["solve"] = solve_measure(lib, abi, L, torch, dev, pos, Lbox, ms)
    if not args.no_lub:
        line["lub"] = lub_measure(lib, abi, L, torch, dev)
    if not args.no_scale and not fp64:
        line["scale"] = scale_measure(lib, abi, L, torch, dev)
    if not args.no_bd:
        line["bd"] = bd_measure(lib, abi, L, torch, dev)
    if not args.no_adjoint:
        line["adjoint"] = adjoint_measure(lib, abi, L)
        line["adjoint"]["fit"] = fit_measure(lib, abi, L)
    if not args.no_batch:
        line["batch"] = batch_measure(lib, abi, L)
    if not args.no_cpu_baseline:
        line["cpu_baseline"], y_or = cpu_baseline(pos, Lbox, x)
        line["rel_err_vs_oracle"] = float(np.linalg.norm(y_timed - y_or) / np.linalg.norm(y_or))
        line["rel_err_vs_oracle_note"] = ("the output of the last timed product against the "
                                          "oracle's FP64 product of the same inputs at the "
                                          "reference split")
    sysm.close()
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-bd", action="store_true", help="skip the Brownian-dynamics leg")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint (VJP) leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the ensemble (batch) leg")
    ap.add_argument("--no-matrix", action="store_true", help="skip the dense-builder leg")
    ap.add_argument("--no-solve", action="store_true", help="skip the iterative-solve leg")
    ap.add_argument("--no-scale", action="store_true",
                    help="skip the larger-N legs of the mixed product")
    ap.add_argument("--no-open", action="store_true",
                    help="skip the free-space (non-periodic) operator leg")
    ap.add_argument("--no-lub", action="store_true", help="skip the lubrication leg")
    ap.add_argument("--n", type=int, default=None,
                    help="override N (smaller cases for profiler captures)")
    args = ap.parse_args()
    if args.n is not None:
        WORKLOAD["n"] = args.n
        WORKLOAD["name"] = f"mob_fts_n{args.n}_phi{WORKLOAD['phi']:.2f}"
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
