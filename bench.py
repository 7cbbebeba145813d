#!/usr/bin/env python3
"""Benchmark: NEMO's per-timestep stencil hot path on the GYRE nn_GYRE=25 basin.

Workload (one "step"): nemo_gpu_stp_hotpath = dyn_spg_ts (phase 1, 37 barotropic
sub-steps in one persistent kernel, phase 3), tsa = 0 + FCT 2nd-order advection of
T and S with on-the-fly transports, rotated iso-neutral laplacian diffusion, and
the implicit vertical diffusion with the salinity clamp, on a 752 x 502 x 31 grid
(11.7 M cells), ln_bench spacing (106 km), rdt = 7200 s. Inputs are the seeded
synthetic GYRE state (analytic T/S + noise, double-gyre flow); they are resident
in HBM and larger than L2 (no L2 flush is needed between steps).

metric: cell-steps/s of the mixed-precision form (FP32 bulk, FP64 barotropic
accumulators); the FP64 plain form is measured on the same inputs and reported
beside it with the SST difference between the two.

--impl reference times the reference's algorithm on the host cores: NEMO cannot
be built here (no Fortran compiler), so that arm runs the oracle (the C FP64
restatement of the reference routines) on a bounded sample of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "nemo-fmi-devel_gb300"))

# the mixed form: FP32 storage and arithmetic; inside the sub-step kernel the five
# barotropic time-filter sums are compensated FP32 pairs (error ~2^-46 of the sum),
# written to FP64 fields once per step
DTYPE_MIXED = "f32 bulk; barotropic time-filter sums as compensated f32 pairs, f64 results"
METRIC = "cell-steps/s, mixed-precision vs FP64 GPU at ≤1e-3 K SST error; % HBM peak"
UNIT = "cell-steps/s"
# algorithmic bytes per 3-D cell of each routine (FP64, FP32-bulk): every 3-D field
# the routine reads or writes counted once; the barotropic sub-steps count 25 2-D
# values per 2-D cell per sub-step (accumulators FP64 in both forms)
ALG_BYTES = {
    "tra_adv": (88, 44),
    "tra_ldf": (88, 44),
    "tra_zdf": (64, 32),
    "dyn_spg_ts_3d": (80, 40),
    "dyn_spg_ts_substep_2d": (200, 140),
}
# the shelf workload (z* variable volume, partial steps) adds the 3-D scale factors
# each routine reads: tra_adv e3u_n e3v_n e3t_b e3t_n e3t_a (5), tra_ldf e3u_n e3v_n
# e3w_n e3t_n (4), tra_zdf e3t_b e3t_n e3t_a e3w_n (4), dyn_spg_ts e3u_n e3v_n e3f_n (3)
ALG_BYTES_SHELF = {
    "tra_adv": (128, 64),
    "tra_ldf": (120, 60),
    "tra_zdf": (96, 48),
    "dyn_spg_ts_3d": (104, 52),
    "dyn_spg_ts_substep_2d": (200, 140),
}
# fields of the shelf state bound on top of the GYRE hot-path set
SHELF_FIELDS = ("gtsu", "gtsv", "ssh_ib", "e3t_b", "e3t_n", "e3t_a", "e3u_n", "e3v_n", "e3w_n", "e3f_n",
                "ht_n", "hu_n", "hv_n", "r1_hu_n", "r1_hv_n", "hu_b", "hv_b", "r1_hu_b", "r1_hv_b")
# algorithmic 3-D fields per cell of each kernel of the hot path (T and S, transports
# computed on the fly, 1-D e3 profile, eddy diffusivity from the masks): every 3-D
# array the kernel reads or writes, counted once; times the element size
KERNEL_FIELDS = {
    "fct_a": 17,     # read un vn wn, tb(2) tn(2); write ta(2) zwi(2) ax(2) ay(2) az(2)
    "fct_b": 14,     # read tb(2) zwi(2) ax(2) ay(2) az(2); write betup(2) betdo(2)
    "fct_c": 20,     # read ax ay az betup betdo (x2), zftu zftv ztfw (x2); ta(2) read+write
    "iso_flux": 14,  # read tb(2) uslp vslp wslpi wslpj; write ah_wslp2 akz, zftu zftv ztfw (x2)
    "iso_flux_tma": 14,  # the same kernel with TMA-staged tracer planes
    "fct_fused": 15,     # read un vn wn tb(2) tn(2), zftu zftv ztfw (x2); write ta(2)
    "fct_a_tma": 17,     # the stage-a / stage-b kernels with TMA-staged planes
    "fct_b_tma": 14,
    "zdf_imp": 8,    # read avt ah_wslp2 tb(2); ta(2) read+write
    "spg_p1a": 2,    # read ua va (column sums; their removal from ua, va is done by phase 3)
    "spg_p3": 8,     # ua va un vn read+write
}
# per 2-D cell, bytes (FP64, FP32-bulk) of the 2-D kernels
KERNEL_BYTES_2D = {
    "spg_p1b": (232, 152),  # ~20 bulk 2-D values + 5 FP64 sums zeroed + 3 ring levels written
}


# DRAM bytes (read + write) per launch from one ncu capture of the DRAM counters of
# this workload's nn_GYRE=15 case, scaled to nn_GYRE=25 by the cell ratio (every
# kernel's traffic is proportional to its cells).
# (kernel, precision, nn_GYRE) -> bytes
TRAFFIC = {(k, "mixed", 25): v * 1e6 for k, v in {
    "spg_p2": 59.1, "iso_flux_tma": 548.6, "fct_c": 901.6, "fct_a_tma": 680.1, "fct_b_tma": 592.6, "zdf_imp": 277.5,
    "spg_p3": 219.6, "spg_p1a": 96.7, "spg_p1b": 36.2}.items()}
TRAFFIC_SOURCE = "ncu dram__bytes_read.sum + dram__bytes_write.sum, nn_GYRE=15 capture scaled by cells"


# FP64 operations (DADD + DMUL + 2 x DFMA thread instructions) and FP64 divisions per
# launch of the FP64 kernels, from one ncu capture at nn_GYRE=15, scaled to the
# workload by cells: (kernel, nn_GYRE) -> (flops, divisions)
FP64_OPS = {}
FP64_OPS_SOURCE = None


def fp64_kernels(kt, nsteps, cells, n2, icycle, nn, shelf):
    """Per-kernel event time of the FP64 step, its algorithmic GB/s against the copy
    bandwidth, and (where the ncu count exists) its FP64 FLOP/s."""
    hbm, _ = peaks()
    out = {}
    for name, (kms, nl) in kt.items():
        us = 1e3 * kms / max(nl, 1)
        if name == "spg_p2":
            kb = ALG_BYTES["dyn_spg_ts_substep_2d"][0] * icycle * n2
        elif name in KERNEL_BYTES_2D:
            kb = KERNEL_BYTES_2D[name][0] * n2
        elif shelf:
            kb = 0
        else:
            kb = KERNEL_FIELDS.get(name, 0) * 8 * cells
        e = {"us": us, "launches_per_step": nl / nsteps, "alg_bytes": kb,
             "alg_GBps": kb / (us / 1e6) / 1e9 if kb and us > 0 else None,
             "frac": kb / (us / 1e6) / 1e9 / hbm if kb and us > 0 else None}
        ops = FP64_OPS.get((name, nn))
        if ops:
            e["fp64_tflops"] = ops[0] / (us / 1e6) / 1e12
            e["fp64_divisions_per_s"] = ops[1] / (us / 1e6)
            e["fp64_ops_source"] = FP64_OPS_SOURCE
        out[name] = e
    return out


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling (every 20 ms) during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        time.sleep(0.05)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=10)
        except Exception:
            self.proc.kill()
            out = ""
        rows = [[x.strip() for x in ln.split(",")] for ln in out.splitlines() if ln.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [v for v in (num(r[1]) for r in rows) if v is not None]
        mx = [v for v in (num(r[2]) for r in rows) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def build_case(nn, nmem, seed, workload="gyre", shelf_grid=(1000, 1200)):
    if workload == "shelf":  # synthetic shelf, 56 z* levels (1000 x 1200 by default)
        from nemo_gpu import shelf
        dom = shelf.domain(shelf_grid[0], shelf_grid[1], 56, seed=seed)
        nam = shelf.namelist()
        states = [shelf.state(dom, nam, seed=seed, member=m) for m in range(nmem)]
        return dom, nam, states
    from nemo_gpu import gyre
    dom = gyre.domain(nn)
    nam = gyre.namelist()
    states = [gyre.state(dom, nam, seed=seed, member=m) for m in range(nmem)]
    return dom, nam, states


def config_dict(args, dom, nam, icycle, nn_baro, world):
    """The workload's configuration, the same dict in both arms of the benchmark."""
    cells = dom["jpi"] * dom["jpj"] * dom["jpk"] * args.members
    return {"workload": workload_name(args), "grid": [dom["jpi"], dom["jpj"], dom["jpk"]],
            "members": args.members, "cells": cells, "icycle": icycle, "nn_baro": nn_baro,
            "rdt": nam["rn_rdt"], "ln_bench": args.workload == "gyre",
            "l2": ("inputs larger than L2 (129 MB), no flush" if cells * 4 * 20 > 129e6
                   else "inputs smaller than L2 (129 MB), no flush"),
            "parallelism": f"replicas x{world}"}


def cpu_model():
    """The host CPU's model name (lscpu), for the CPU figures."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def workload_name(args):
    if args.workload == "shelf":
        nx, ny = args.shelf_grid
        return (f"synthetic shelf {nx}x{ny}x56 hot path step (dyn_spg_ts z* flux form + FCT 4/4 + iso ldf "
                "with partial steps + zdf)")
    return f"GYRE nn_GYRE={args.nn} hot path step (dyn_spg_ts + FCT + iso ldf + zdf)"


HOT_3D = ("un", "vn", "wn", "ua", "va", "avt", "uslp", "vslp", "wslpi", "wslpj")
HOT_2D = ("sshn", "un_b", "vn_b", "ub_b", "vb_b", "utau", "vtau", "emp")
ACC_2D = ("SSHA", "UA_B", "VA_B", "UN_ADV", "VN_ADV", "UB2_B", "VB2_B", "UN_BF", "VN_BF")


def make_ctx(dom, nam, states, prec, stream):
    """A context with every hot-path field bound to device tensors holding the state."""
    import numpy as np
    import torch
    from nemo_gpu import api
    ctx = api.Context(dom, nam, nmembers=len(states), prec=prec, stream=stream)
    dev = {}

    def put(name, arrays, fp64=False):
        t = ctx.to_device(arrays, dtype=torch.float64 if fp64 else None)
        dev[name] = t
        ctx.bind(name, t)

    put("TSB", [s["tsb"] for s in states])
    put("TSN", [s["tsn"] for s in states])
    put("TSA", [np.zeros_like(s["tsb"]) for s in states])
    for n in HOT_3D:
        put(n.upper(), [s[n] for s in states])
    for n in ("ub", "vb", "sshb"):
        put(n.upper(), [s[n] for s in states])
    for n in HOT_2D:
        put(n.upper(), [s[n] for s in states])
    put("RCDU_BOT", [s["rcdu_bot"] for s in states])
    z3 = [np.zeros_like(s["avt"]) for s in states]
    put("AH_WSLP2", z3)
    put("AKZ", z3)
    z2 = [np.zeros_like(s["sshn"]) for s in states]
    for n in ACC_2D:  # the restart fields of a run in progress where the state has them
        put(n, [s[n.lower()] for s in states] if n.lower() in states[0] else z2, fp64=True)
    for n in SHELF_FIELDS:
        if n in states[0]:
            put(n.upper(), [s[n] for s in states])
    return ctx, dev


def full_gyre(dom, nam, states):
    """The namelist and the states of the full GYRE step (gyre.full_physics)."""
    from nemo_gpu import gyre
    out = [gyre.full_physics(dom, nam, st) for st in states]
    return out[0][0], [st for _, st in out]


def bind_full(ctx, dev, states):
    """Bind the fields of the full GYRE step (besides make_ctx's)."""
    import numpy as np
    import torch
    from nemo_gpu import gyre
    for n in gyre.FULL_3D + gyre.FULL_2D:
        t = ctx.to_device([s[n] for s in states])
        dev[n.upper()] = t
        ctx.bind(n.upper(), t)
    t = torch.from_numpy(np.concatenate([np.asarray(s["nmln"], dtype=np.int32).ravel(order="F")
                                         for s in states])).cuda()
    dev["NMLN"] = t
    ctx.bind("NMLN", t)


def ten_days(dom, nam, states, stream, nsteps=120):
    """The mixed form against FP64 after ten model days (120 steps of rdt = 7200 s) of
    the full GYRE step (nemo_gpu_stp_model with GYRE's physics) from an Euler start on
    the same state: RMS over wet points and max of |mixed - FP64| for T, S, SST, SSS,
    SSH, U, V."""
    import numpy as np
    nam = dict(nam, neuler=0)
    nam, states = full_gyre(dom, nam, states)
    # the FP64 step from the same state rounded to FP32: how far the model's own
    # sensitivity (convective and closure thresholds) carries a 6e-8 perturbation
    rounded = [{k: (np.asfortranarray(v.astype(np.float32).astype(np.float64))
                    if isinstance(v, np.ndarray) and v.dtype == np.float64 else v) for k, v in st.items()}
               for st in states]
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    out = {}
    for prec, sts in (("fp64", states), ("mixed", states), ("fp64_rounded", rounded)):
        ctx, dev = make_ctx(dom, nam, sts, prec.split("_")[0], stream)
        bind_full(ctx, dev, sts)
        for kt in range(1, nsteps + 1):
            ctx.stp_model(kt)
        ctx.synchronize()
        get = lambda n, sh: np.asarray(ctx.to_host(dev[n], sh))
        out[prec] = {"T": get("TSN", (jpi, jpj, jpk, 2))[..., 0], "S": get("TSN", (jpi, jpj, jpk, 2))[..., 1],
                     "U": get("UN", (jpi, jpj, jpk)), "V": get("VN", (jpi, jpj, jpk)), "SSH": get("SSHN", (jpi, jpj))}
        ctx.close()
        del dev
    tm = np.arange(1, jpk + 1)[None, None, :] <= dom["k_bot"][:, :, None]
    res = {"steps": nsteps, "model_days": nsteps * nam["rn_rdt"] / 86400.0,
           "step": "nemo_gpu_stp_model with GYRE's physics: rab_3d + bn2, zdf_phy (TKE, evd), zdf_mxl, "
                   "eos_insitu + ldf_slp, dyn_keg + dyn_zad + vor_ene + dyn_ldf_lap, EOS-80 + dyn_hpg, "
                   "dyn_spg_ts, wzv, dyn_zdf (implicit viscosity), tra_sbc + tra_qsr, the hot path, "
                   "tra_nxt, dyn_nxt, ssh_swp, stp_ctl",
           "forcing": "GYRE's analytic fluxes formed on the device every step (usrdef_sbc)",
           "fp64_rounded": "the FP64 step started from the same state rounded to FP32, against the FP64 step: "
                           "the model's own sensitivity, a floor for any FP32-storage form"}
    for n, sel in (("T", None), ("S", None), ("SST", "T"), ("SSS", "S"), ("U", None), ("V", None), ("SSH", None)):
        b = out["fp64"][sel or n]
        if n in ("SST", "SSS"):
            b, m = b[:, :, 0], tm[:, :, 0]
        elif n == "SSH":
            m = tm[:, :, 0]
        else:
            m = tm
        res[n] = {"range": float(np.abs(b[m]).max())}
        for arm in ("mixed", "fp64_rounded"):
            a = out[arm][sel or n]
            if n in ("SST", "SSS"):
                a = a[:, :, 0]
            d = (a - b)[m]
            key = "" if arm == "mixed" else "_fp64_rounded"
            res[n]["rms" + key] = float(np.sqrt(np.mean(d * d)))
            res[n]["max" + key] = float(np.abs(d).max())
    return res


def time_steps(ctx, stream, steps, kt0, dev_index):
    import torch
    from nemo_gpu import dist
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier(dev_index)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        e0.record(stream)
        for s in range(steps):
            ctx.stp_hotpath(kt0 + s)
        e1.record(stream)
    torch.cuda.synchronize()
    dist.barrier(dev_index)
    ctx.synchronize()
    return e0.elapsed_time(e1)


def run_gpu(args):
    import numpy as np
    import torch
    from nemo_gpu import dist
    rank, world = dist.init("nccl")
    _, _, local = dist.env_rank()
    torch.cuda.set_device(local)
    dom, nam, states = build_case(args.nn, args.members, seed=100 + rank, workload=args.workload,
                                   shelf_grid=args.shelf_grid)
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    cells = jpi * jpj * jpk * args.members
    stream = torch.cuda.Stream()
    out = {}
    # ---------------------------------------------------------------- mixed (headline)
    ctx, dev = make_ctx(dom, nam, states, args.prec, stream)
    icycle, nn_baro, _ = ctx.spg_info()
    kt0 = 5
    for w in range(args.warmup):
        ctx.stp_hotpath(kt0 + w)
    ctx.synchronize()
    # the launch shapes of the 32-wide kernels, chosen by the autotuner on this state
    # (it puts back every field it writes), then one untimed step to capture the graph
    shape = None
    if not args.no_autotune:
        ctx.autotune(kt0 + 700, nrep=3)
        shape = {k: v for k, v in ctx.launch_shape().items()
                 if k in ("fct_a", "fct_b", "fct_c", "iso_flux", "zdf_imp", "spg_cor", "spg_p1a", "spg_p1b",
                          "spg_p3")}
        ctx.stp_hotpath(kt0 + args.warmup)
        ctx.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    ms = time_steps(ctx, stream, args.steps, kt0 + args.warmup + 1, local)
    ck = clocks.stop()
    ck["window_ms"] = ms
    ms_max = dist.max_over_ranks(ms, device=f"cuda:{local}")
    ms_step = ms_max / args.steps
    value = cells * world * args.steps / (ms_max / 1e3)
    # per-routine and per-kernel timing (CUDA events on the context's stream)
    ctx.set_timing(True)
    ntime = max(3, min(args.steps, 10))
    for s in range(ntime):
        ctx.stp_hotpath(kt0 + 1000 + s)
    ctx.synchronize()
    rt, ncalls = ctx.get_timing()
    kt_ = ctx.get_kernel_timing()
    ctx.set_timing(False)
    rt = {k: v / max(ncalls, 1) for k, v in rt.items()}
    launches_per_step = sum(n for _, n in kt_.values()) / ntime
    sst_mixed = ctx.to_host(dev["TSA"], (jpi, jpj, jpk, 2))
    # ---------------------------------------------------------------- FP64 arm
    fp64 = None
    if not args.no_fp64 and args.prec == "mixed":
        ctx64, dev64 = make_ctx(dom, nam, states, "fp64", stream)
        for w in range(2):
            ctx64.stp_hotpath(kt0 + w)
        ctx64.synchronize()
        k64 = max(2, args.steps // 4)
        ms64 = dist.max_over_ranks(time_steps(ctx64, stream, k64, kt0 + 2, local), device=f"cuda:{local}")
        ctx64.set_timing(True)
        for s in range(3):
            ctx64.stp_hotpath(kt0 + 1000 + s)
        ctx64.synchronize()
        rt64, n64 = ctx64.get_timing()
        kt64 = ctx64.get_kernel_timing()
        ctx64.set_timing(False)
        # the same step on the same inputs in both forms: SST (T at level 1) difference
        for c_, d_ in ((ctx, dev), (ctx64, dev64)):
            for n in ("UA", "VA", "UN", "VN"):
                d_[n].copy_(c_.to_device([s[n.lower()] for s in states]))
            for n in ACC_2D:
                if n.lower() in states[0]:
                    d_[n].copy_(c_.to_device([s[n.lower()] for s in states], dtype=torch.float64))
                else:
                    d_[n].zero_()
            c_.stp_hotpath(kt0 + 5000)
            c_.synchronize()
        a32 = ctx.to_host(dev["TSA"], (jpi, jpj, jpk, 2))
        a64 = ctx64.to_host(dev64["TSA"], (jpi, jpj, jpk, 2))
        if isinstance(a32, list):
            a32, a64 = a32[0], a64[0]
        tm = dom["k_bot"] > 0
        sst_err = float(np.abs(a32[:, :, 0, 0] - a64[:, :, 0, 0])[tm].max())
        sss_err = float(np.abs(a32[:, :, 0, 1] - a64[:, :, 0, 1])[tm].max())
        fp64 = {"value": cells * world * k64 / (ms64 / 1e3), "ms_per_step": ms64 / k64,
                "routine_ms": {k: v / max(n64, 1) for k, v in rt64.items()},
                "kernels": fp64_kernels(kt64, 3, cells, n2=jpi * jpj * args.members, icycle=icycle, nn=args.nn,
                                        shelf=args.workload == "shelf"),
                "sst_abs_err_1step_K": sst_err, "sss_abs_err_1step_psu": sss_err}
        ctx64.close()
        del dev64
        if not args.no_ten_days and args.workload == "gyre" and rank == 0:
            fp64["ten_days"] = ten_days(dom, nam, states[:1], stream)
    # ---------------------------------------------------------------- e2e (host buffers, C ABI)
    e2e = None
    if not args.no_e2e:
        # in the order the previous step releases them (the upload of a field waits for
        # the last part of the previous step that reads it): dyn_spg_ts's own fields,
        # the slopes (iso-neutral fluxes), the velocities and tn (FCT), then the rest;
        # downloads of what dyn_spg_ts writes first (they start when it ends)
        shelf = [n.upper() for n in SHELF_FIELDS if n in states[0]]
        late = ("GTSU", "GTSV", "E3T_B", "E3T_N", "E3T_A", "E3U_N", "E3V_N", "E3W_N", "E3F_N")
        ins = (["UA", "VA"] + [n.upper() for n in HOT_2D if n not in ("un_b", "vn_b")] + ["UN_B", "VN_B", "RCDU_BOT"]
               + [n for n in shelf if n not in late]
               + ["USLP", "VSLP", "WSLPI", "WSLPJ"] + [n for n in shelf if n in ("GTSU", "GTSV")]
               + ["UN", "VN", "WN", "TSN", "TSB", "AVT"] + [n for n in shelf if n in late[2:]])
        assert sorted(ins) == sorted(set(ins))
        outs = ["UA", "VA", "UN", "VN"] + list(ACC_2D) + ["TSA", "AH_WSLP2"]
        host = {}
        for n in set(ins + outs):
            host[n] = torch.empty(dev[n].numel(), dtype=dev[n].dtype, pin_memory=True)
            host[n].copy_(dev[n].cpu())
        bi = sum(host[n].numel() * host[n].element_size() for n in ins)
        bo = sum(host[n].numel() * host[n].element_size() for n in outs)
        ke = max(2, args.steps // 2)
        for n in ins:  # one untimed round (the context makes its staging buffers here)
            ctx.upload(n, host[n])
        ctx.stp_hotpath(kt0 + 8999)
        for n in outs:
            ctx.download(n, host[n])
        ctx.synchronize()
        t0 = time.perf_counter()
        for s in range(ke):
            for n in ins:
                ctx.upload(n, host[n])
            ctx.stp_hotpath(kt0 + 9000 + s)
            for n in outs:
                ctx.download(n, host[n])
        ctx.synchronize()
        wall = time.perf_counter() - t0
        wms = dist.max_over_ranks(1e3 * wall, device=f"cuda:{local}")
        e2e = {"value": cells * world * ke / (wms / 1e3), "unit": UNIT, "h2d_bytes_per_step": bi,
               "d2h_bytes_per_step": bo, "ms_per_step": wms / ke,
               "timer": "host wall clock from the first upload to the synchronize after the last download",
               "host_buffers": "pinned; nemo_gpu_field_upload/download through the C ABI"}
    # ---------------------------------------------------------------- the full GYRE step
    model = None
    if not args.no_model and args.workload == "gyre":
        km = max(3, args.steps // 5)
        ms_m, kt_m = model_step(dom, nam, states, args.prec, stream, km, 3, local)
        model = {"value": cells * world / (ms_m / 1e3), "unit": UNIT, "ms_per_step": ms_m, "steps": km,
                 "step": "nemo_gpu_stp_model with GYRE's physics (EOS-80, TKE + evd, slopes from the tracers, "
                         "momentum trends, implicit vertical viscosity, surface forcing, stp_ctl), "
                         "device-resident, CUDA events",
                 "launches_per_step": sum(v["launches"] for v in kt_m.values()),
                 "kernels_us_per_step": {k: v["us"] * v["launches"] for k, v in
                                         sorted(kt_m.items(), key=lambda kv: -kv[1]["us"] * kv[1]["launches"])}}
    # ---------------------------------------------------------------- roofline
    hbm, src = peaks()
    b = 1 if args.prec == "mixed" else 0
    AB = ALG_BYTES_SHELF if args.workload == "shelf" else ALG_BYTES
    per_cell = {"tra_adv": AB["tra_adv"][b], "tra_ldf": AB["tra_ldf"][b],
                "tra_zdf": AB["tra_zdf"][b],
                "dyn_spg_ts": AB["dyn_spg_ts_3d"][b]
                + AB["dyn_spg_ts_substep_2d"][b] * icycle / jpk}
    es = 4 if args.prec == "mixed" else 8
    n2 = jpi * jpj * args.members

    def kernel_bytes(name):
        if name == "spg_p2":  # every 2-D value of every sub-step (L2-resident working set)
            return ALG_BYTES["dyn_spg_ts_substep_2d"][b] * icycle * n2
        if name in KERNEL_BYTES_2D:
            return KERNEL_BYTES_2D[name][b] * n2
        if name in ("iso_akz_edges", "iso_msc_edges"):  # edge columns only: ah_wslp2, akz
            return 2 * es * (2 * jpi + 2 * jpj) * jpk * args.members
        if args.workload == "shelf":  # per-kernel models are for the GYRE kernels (1-D e3)
            return 0
        return KERNEL_FIELDS.get(name, 0) * es * cells

    kernels = {}
    for name, (kms, nl) in kt_.items():
        us = 1e3 * kms / max(nl, 1)
        kb = kernel_bytes(name)
        kernels[name] = {"us": us, "launches_per_step": nl / ntime, "alg_bytes": kb,
                         "alg_GBps": kb / (us / 1e6) / 1e9 if kb and us > 0 else None,
                         "frac": kb / (us / 1e6) / 1e9 / hbm if kb and us > 0 else None}
    modelled = [k for k in kernels if kernels[k]["alg_bytes"]]
    top = max(modelled or kernels, key=lambda k: kernels[k]["us"])
    achieved = kernels[top]["alg_GBps"]
    alg_bytes = kernels[top]["alg_bytes"]
    routines = {k: {"ms": rt[k], "alg_GBps": per_cell[k] * cells / (rt[k] / 1e3) / 1e9,
                    "frac": per_cell[k] * cells / (rt[k] / 1e3) / 1e9 / hbm} for k in rt if rt[k] > 0.01}
    step_bytes = sum(per_cell[k] for k in per_cell) * cells
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPE_MIXED if args.prec == "mixed" else "f64",
        "data": "synthetic: seeded GYRE analytic state (no reference data files exist)" if args.workload == "gyre"
        else "synthetic: seeded shelf (lognormal bathymetry, z*, partial steps); no reference data files exist",
        "config": config_dict(args, dom, nam, icycle, nn_baro, world),
        "resident_GB": sum(t.numel() * t.element_size() for t in dev.values()) / 1e9,
        "launch_shape": ({k: f"32x{v}" for k, v in shape.items()} if shape else "32x4 (not tuned)"),
        "clocks": ck, "gpu_launches": int(round(launches_per_step * args.steps)),
        "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm if achieved else None, "traffic": TRAFFIC.get((top, args.prec, args.nn)),
                     "traffic_source": TRAFFIC_SOURCE if (top, args.prec, args.nn) in TRAFFIC else None,
                     "peak_source": src, "alg_bytes_per_launch": alg_bytes,
                     "duration_us": kernels[top]["us"]},
        "kernels": kernels,
        "routines": routines,
        "step_alg_GBps": step_bytes / (ms_step / 1e3) / 1e9,
        "e2e": e2e, "fp64": fp64, "model_step": model,
    }
    if fp64:
        res["speedup_vs_fp64"] = value / fp64["value"]
    if rank == 0 and world == 1 and not args.no_cpu:
        res["cpu_baseline"] = cpu_baseline(dom, nam, states[0], budget_s=args.cpu_budget, what=workload_name(args))
    ctx.close()
    if rank == 0:
        print(json.dumps(res))


class OracleStep:
    """The oracle (C FP64 restatement of the reference routines) bound to one
    member's state of the workload, stepping the hot path on the host cores."""

    def __init__(self, dom, nam, st):
        import numpy as np
        from oracle import ora
        self.o = o = ora.Oracle(dom, nam)
        self.keep = keep = {}
        for n in ("tsb", "tsn") + HOT_3D + ("ub", "vb", "sshb") + HOT_2D:
            keep[n] = np.array(st[n], order="F", copy=True)
            o.bind(n.upper(), keep[n])
        keep["rc"] = np.array(st["rcdu_bot"], order="F", copy=True)
        o.bind("RCDU_BOT", keep["rc"])
        for n in SHELF_FIELDS:
            if n in st:
                keep[n] = np.array(st[n], order="F", copy=True)
                o.bind(n.upper(), keep[n])
        keep["tsa"] = np.zeros_like(st["tsb"], order="F")
        o.bind("TSA", keep["tsa"])
        for n in ("AH_WSLP2", "AKZ"):
            keep[n] = np.zeros_like(st["avt"], order="F")
            o.bind(n, keep[n])
        for n in ACC_2D:
            keep[n] = (np.array(st[n.lower()], order="F", copy=True) if n.lower() in st
                       else np.zeros(st["sshn"].shape, order="F"))
            o.bind(n, keep[n])
        self.kt = 5

    def step(self):
        self.o.stp_hotpath(self.kt)
        self.kt += 1

    def close(self):
        self.o.close()


def cpu_baseline(dom, nam, st, budget_s=20.0, what="GYRE nn_GYRE=25 workload"):
    """The oracle on the host cores: all cores (OpenMP) on a bounded sample of full
    steps, and one core on one step. The oracle's work arrays are allocated on the
    first (untimed) step and reused after it."""
    from oracle import ora
    ncores = os.cpu_count()
    cells = dom["jpi"] * dom["jpj"] * dom["jpk"]
    s = OracleStep(dom, nam, st)
    ora.set_threads(ncores)
    s.step()  # untimed: first touch of the work arrays
    t0 = time.perf_counter()
    n = 0
    while True:
        s.step()
        n += 1
        if time.perf_counter() - t0 > 0.7 * budget_s or n >= 50:
            break
    dt = time.perf_counter() - t0
    ora.set_threads(1)
    t1 = time.perf_counter()
    s.step()
    dt1 = time.perf_counter() - t1
    ora.set_threads(ncores)
    s.close()
    return {"value": cells * n / dt, "unit": UNIT, "cores": ncores, "kind": "port",
            "sample": f"{n} full hot-path steps of the same {what} (FP64 oracle, OpenMP, {ncores} threads) "
                      f"after one untimed step",
            "single_thread": {"value": cells / dt1, "unit": UNIT, "cores": 1, "sample": "one full step"},
            "cpu_model": cpu_model(), "build": "gcc -O3 -ffp-contract=off -fno-fast-math -fopenmp"}


def run_reference(args):
    """The reference arm: the oracle on the host cores, --warmup untimed full steps
    then exactly --steps timed full steps of the same workload (rank 0 only)."""
    from nemo_gpu import dist
    from oracle import ora
    rank, world = dist.init("gloo")
    if rank != 0:
        return
    dom, nam, states = build_case(args.nn, args.members, seed=100, workload=args.workload,
                                   shelf_grid=args.shelf_grid)
    ncores = os.cpu_count()
    ora.set_threads(ncores)
    members = [OracleStep(dom, nam, st) for st in states]  # one oracle per member, stepped in turn
    icycle, nn_baro, _ = members[0].o.spg_info()
    for _ in range(args.warmup):
        for s in members:
            s.step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for s in members:
            s.step()
    dt = time.perf_counter() - t0
    for s in members:
        s.close()
    cells = dom["jpi"] * dom["jpj"] * dom["jpk"] * args.members
    value = cells * args.steps / dt
    cb = {"value": value, "unit": UNIT, "cores": ncores, "kind": "port",
          "sample": f"{args.steps} full hot-path steps after {args.warmup} untimed ones (FP64 oracle, OpenMP, "
                    f"{ncores} threads)", "cpu_model": cpu_model(),
          "build": "gcc -O3 -ffp-contract=off -fno-fast-math -fopenmp"}
    res = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic: seeded GYRE analytic state (no reference data files exist)" if args.workload == "gyre"
           else "synthetic: seeded shelf (lognormal bathymetry, z*, partial steps); no reference data files exist",
           "config": config_dict(args, dom, nam, icycle, nn_baro, world),
           "cpu_baseline": cb,
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "NEMO (Fortran) cannot be built in this environment; the reference arm runs the C FP64 "
                   "restatement of the same routines (oracle/) on the host cores"}
    print(json.dumps(res))


def model_step(dom, nam, states, prec, stream, steps, warmup, local):
    """Device time of the full GYRE step (nemo_gpu_stp_model with GYRE's physics) on
    resident fields: ms per step, the kernels of one step and their launches."""
    import torch
    from nemo_gpu import dist
    nam, states = full_gyre(dom, dict(nam, neuler=0), states)
    ctx, dev = make_ctx(dom, nam, states, prec, stream)
    bind_full(ctx, dev, states)
    for w in range(warmup):
        ctx.stp_model(1 + w)
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier(local)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        e0.record(stream)
        for s in range(steps):
            ctx.stp_model(1 + warmup + s)
        e1.record(stream)
    torch.cuda.synchronize()
    ms = dist.max_over_ranks(e0.elapsed_time(e1), device=f"cuda:{local}")
    ctx.set_timing(True)
    for s in range(3):
        ctx.stp_model(5000 + s)
    ctx.synchronize()
    kt = {k: {"us": 1e3 * v[0] / v[1], "launches": v[1] / 3} for k, v in ctx.get_kernel_timing().items()}
    ctx.set_timing(False)
    ctx.close()
    return ms / steps, kt


def run_model(args):
    """The full GYRE step (nemo_gpu_stp_model with GYRE's physics) on GYRE
    nn_GYRE=--nn, in --prec, device-resident."""
    import torch
    from nemo_gpu import dist
    rank, world = dist.init("nccl")
    _, _, local = dist.env_rank()
    torch.cuda.set_device(local)
    dom, nam, states = build_case(args.nn, args.members, seed=100 + rank)
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    cells = jpi * jpj * jpk * args.members
    stream = torch.cuda.Stream()
    ms_step, kt = model_step(dom, nam, states, args.prec, stream, args.steps, args.warmup, local)
    ms = ms_step * args.steps
    if rank == 0:
        print(json.dumps({
            "metric": "cell-steps/s of the full GYRE step (nemo_gpu_stp_model with GYRE's physics)",
            "value": cells * world * args.steps / (ms / 1e3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPE_MIXED if args.prec == "mixed" else "f64",
            "data": "synthetic: seeded GYRE analytic state",
            "config": {"workload": f"GYRE nn_GYRE={args.nn} full model step", "grid": [jpi, jpj, jpk],
                       "members": args.members, "cells": cells},
            "gpu_launches": int(round(sum(v["launches"] for v in kt.values()) * args.steps)), "kernels": kt}))


def run_window(args):
    """C4: gradient of the SST cost of a 48-step FP64 tracer window on GYRE
    nn_GYRE=10 (forward sweep + checkpointed reverse sweep, checkpoints every 8)."""
    import numpy as np
    import torch
    from nemo_gpu import adjoint, api, gyre
    nn, nwin, every = args.nn if args.nn != 25 else 10, 48, 8
    dom = gyre.domain(nn)
    nam = gyre.namelist(neuler=0)
    st = gyre.state(dom, nam, seed=100)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        ctx = api.Context(dom, nam, nmembers=1, prec="fp64", stream=stream)
        put = lambda n, a: (ctx.bind(n, ctx.to_device(a)), ctx.bound[n])[1]
        for n in ("avt", "uslp", "vslp", "wslpi", "wslpj"):
            put(n.upper(), st[n])
        z3 = np.zeros_like(st["avt"])
        put("AH_WSLP2", z3)
        put("AKZ", z3)
        for n in ("TSB", "TSN", "TSA"):
            put(n, np.zeros_like(st["tsb"]))
        un, vn, wn = (ctx.to_device(st[k]) for k in ("un", "vn", "wn"))
        zun, zvn, zwn = (torch.empty_like(un) for _ in range(3))
        ctx.tra_adv_trp(un, vn, wn, zun, zvn, zwn)
        win = adjoint.TracerWindow(ctx, zun, zvn, zwn, nwin, every=every)
        t0 = ctx.to_device(st["tsn"])
        jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
        tm = torch.from_numpy(np.ascontiguousarray((st["tsn"][:, :, 0, 0] != 0).T.astype(np.float64))).cuda()
        target = ctx.to_device(st["tsn"]).view(2, jpk, jpj, jpi)[0, 0][None] + 0.1

        def gradient():
            _, tsn = win.forward(t0, t0)
            _, g = adjoint.sst_cost(tsn, target, tm, (jpi, jpj, jpk))
            return win.adjoint(torch.zeros_like(g), g)

        for _ in range(args.warmup):
            gradient()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        torch.cuda.synchronize()
        e[0].record(stream)
        for _ in range(args.steps):
            win.forward(t0, t0)
        e[1].record(stream)
        torch.cuda.synchronize()
        e[2].record(stream)
        for _ in range(args.steps):
            ab, an = gradient()
        e[3].record(stream)
        torch.cuda.synchronize()
    fwd_ms, grad_ms = e[0].elapsed_time(e[1]) / args.steps, e[2].elapsed_time(e[3]) / args.steps
    cells = jpi * jpj * jpk
    # launches per gradient: forward and recomputed steps (FCT a, b, c; iso flux, div,
    # edges; zdf; nxt = 8 each), adjoint steps (nxt, zdf, iso x3, fct = 6)
    launches = args.steps * (nwin * 8 * 2 + nwin * 6)
    res = {"metric": "cell-steps/s of the adjoint window gradient (forward + checkpointed reverse sweep)",
           "value": cells * nwin / (grad_ms * 1e-3), "unit": "cell-steps/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": grad_ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic: seeded GYRE analytic state",
           "config": {"workload": f"GYRE nn_GYRE={nn} FP64 tracer window, {nwin} steps, checkpoints every {every}, "
                                  "J = sum (SST - target)^2", "cells": cells, "window_steps": nwin,
                      "l2": "inputs (2 x 31 MB per state) below L2; no flush"},
           "forward_sweep_ms": fwd_ms, "gradient_over_forward": grad_ms / fwd_ms, "gpu_launches": launches}
    print(json.dumps(res))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--prec", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--nn", type=int, default=25)
    ap.add_argument("--workload", default="gyre", choices=["gyre", "shelf", "window", "model"],
                    help="gyre: GYRE nn_GYRE=--nn (the headline); shelf: the 1000x1200x56 z* shelf; "
                         "window: the gradient of a 48-step FP64 tracer window (nn_GYRE=10); "
                         "model: the model step (the hot path closed into a time step)")
    ap.add_argument("--shelf-grid", type=int, nargs=2, default=[1000, 1200], metavar=("NX", "NY"),
                    help="horizontal size of the shelf workload (a smaller one for profiler captures)")
    ap.add_argument("--members", type=int, default=1)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default 32 x 4 launch shapes")
    ap.add_argument("--no-ten-days", action="store_true", help="skip the ten-day mixed-vs-FP64 divergence")
    ap.add_argument("--no-model", action="store_true", help="skip the timing of the full GYRE step")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "window":
        run_window(args)
    elif args.workload == "model":
        run_model(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
