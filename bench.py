"""Benchmark of the forward path on the 3D 30k-node cylinder (100 MHz).

One step = one request through tg_forward_path: assembly + IC(0) factor,
80 forward and 80 adjoint source solves (BiCGSTAB + ICH), ProjectAll (linear
and log) and the full nodal Jacobian (12800 x 61620).  The metric is
source-solves/s (forward + adjoint) of whole requests, so every solve carries
its share of assembly, projection and Jacobian.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--precision mixed|fp64] [--tol T]

--impl reference times the CPU restatement of the reference (oracle/, the
reference's algorithm with threads over sources) on this host's cores, on a
bounded sample of each request, extrapolated to whole requests.
Prints one JSON line on rank 0.
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

UNIT = "source-solves/s"
# DRAM traffic per launch of the dominant kernel (ncu dram__bytes_read.sum +
# dram__bytes_write.sum), captured on a smaller case of the same kernel and
# scaled to the workload by the units one launch processes; the capture
# commands and counters are in profiles/
TRAFFIC = {
    ("c2_cyl30k_fd", "jacobian_oz"): (
        (332.53632e6 + 1653.086e6) * (12800 * 61620) / (12800 * 15008),
        "ncu on the 7504-node cylinder (12800 x 15008 J: read 332.5 MB + write 1653.1 MB), scaled by the J "
        "entries to 12800 x 61620 (profiles/jacobian_oz_kernel_cyl7k_fp64.md)"),
    ("c2_cyl30k_fd", "jacobian_ff"): (
        (179.457792e6 + 1477.513e6) * (12800 * 61620) / (12800 * 15008),
        "ncu on the 7504-node cylinder (12800 x 15008 J: read 179.5 MB + write 1477.5 MB), scaled by the J "
        "entries to 12800 x 61620 (profiles/jacobian_ff_kernel_cyl7k_fp64.md)"),
}
LABELS = {"c0_disc3k_cw": "2D 3.3k-node disc CW", "c1_disc13k_fd": "2D 13k-node disc 100 MHz",
          "c2_cyl30k_fd": "3D 30k-node cylinder 100 MHz", "c3_box250k_fd": "3D 250k-node box 100 MHz",
          "c2s_cyl7k_fd": "3D 7.5k-node cylinder 100 MHz (profiling case)",
          "c3s_box106k_fd": "3D 106k-node box 100 MHz (profiling case)"}


def metric_of(cfg):
    return ("source-solves/s (fwd+adj, whole requests incl. assembly, ProjectAll, Jacobian), " + LABELS[cfg])


def method_of(P):
    return "BICGSTAB" if P.complex else "CG"


def workload_of(P, cfg, n_el, tol, precision, extra=""):
    nq, nm, nqm = P.qm.nQ, P.qm.nM, P.qm.nQM
    kind = "tets" if P.dim == 3 else "triangles"
    cols = 2 * P.n if P.complex else P.n
    return (f"{cfg}: {P.n} nodes, {n_el} {kind}, {'%g MHz' % P.freq_mhz if P.complex else 'CW'}, {nq}+{nm} optodes, "
            f"{method_of(P)}+ICH tol {tol}, {precision}{extra}, nodal Jacobian {2 * nqm}x{cols}")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c2_cyl30k_fd",
                    choices=["c0_disc3k_cw", "c1_disc13k_fd", "c2_cyl30k_fd", "c3_box250k_fd", "c2s_cyl7k_fd",
                             "c3s_box106k_fd"])
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg")
    ap.add_argument("--e2e-slots", type=int, default=2, help="e2e leg: request-server slots")
    ap.add_argument("--no-concurrent", action="store_true",
                    help="skip the leg with two requests on the device at once")
    ap.add_argument("--grid", type=int, default=32,
                    help="grid-basis Jacobian leg: raster points per axis (0: skip)")
    ap.add_argument("--element", action="store_true",
                    help="also time the element-basis Jacobian on the same fields")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--jac", default="fp64", choices=["fp64", "fp32", "fp32acc"],
                    help="Jacobian output: fp64 (FP64-accurate from the FP64 fields), fp32 (FP32 arithmetic), "
                         "fp32acc (FP32 storage of the FP64-accurate sums)")
    ap.add_argument("--cw-tol", type=float, default=1e-10,
                    help="mixed path: componentwise backward-error bound of every solution (0: off)")
    ap.add_argument("--tol", type=float, default=1e-12)
    ap.add_argument("--inner-tol", type=float, default=1e-4, help="mixed path: inner FP32 solve tolerance")
    ap.add_argument("--inner-order", type=int, default=1, help="mixed path: inner IC(0) ordering, 1 colour, 0 natural")
    ap.add_argument("--no-compare", action="store_true", help="skip the FP64 comparison legs")
    ap.add_argument("--inner", default="cocg", choices=["cocg", "bicgstab", "restart"],
                    help="mixed path: FP32 inner process (reliable updates of COCG or BiCGSTAB, or restarts)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--serving", action="store_true",
                    help="run the mixed-mesh request stream through the request server instead")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-stream leg of the default run")
    ap.add_argument("--requests", type=int, default=24, help="serving: requests in the stream")
    ap.add_argument("--rate", type=float, default=20.0, help="serving: mean arrival rate (1/s)")
    ap.add_argument("--slots", type=int, default=4, help="serving: concurrent requests on the device")
    ap.add_argument("--src-max-large", type=int, default=64, help="serving: source cap on the 250k box")
    return ap.parse_args()


def problem(cfg="c2_cyl30k_fd"):
    from toastpp_gb300 import workloads
    return workloads.CONFIGS[cfg]()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                f = [x.strip() for x in out.stdout.strip().split(",")]
                if len(f) >= 7:
                    self.samples.append(f)
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# ---------------------------------------------------------------------------
# CPU legs (oracle port; test infrastructure used here only as the baseline)
# ---------------------------------------------------------------------------
def cpu_request_time(P, nsrc_sample=None, nq_jac_sample=2, threads=None, tol=1e-12):
    """Time one request on the host cores: full assembly + IC factor, a sample of
    the source solves (one per host thread, forward and adjoint) and of the
    Jacobian rows (nq_jac_sample sources x all sampled detectors, the links
    shared by all threads); extrapolate linearly to the whole request.  The
    reference arm and the GPU line's cpu_baseline call this with the same
    arguments."""
    nsrc_sample = nsrc_sample or max(8, os.cpu_count() or 1)
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    m = O.Mesh(P.coords, P.elems)
    cm, ck, ca = O.optical_coefficients(P.mua, P.mus, P.nref)
    omega = P.freq_mhz * 2 * np.pi * 1e-6
    nq, nm = P.qm.nQ, P.qm.nM
    meth = method_of(P)
    dt = np.complex128 if P.complex else np.float64
    t0 = time.perf_counter()
    val = m.assemble(cm, ck, ca, omega, P.complex)
    O.ic_factor(m.rowptr, m.colidx, val)
    t_reset = time.perf_counter() - t0
    rng = np.random.default_rng(7)
    qs = rng.choice(nq, size=min(nsrc_sample, nq), replace=False)
    ms = rng.choice(nm, size=min(nsrc_sample, nm), replace=False)
    qvec = np.stack([m.qvec_gaussian(P.qm.Q[i], P.qwidth) for i in range(nq)]).astype(dt)
    mvec = np.stack([m.qvec_gaussian(P.qm.M[i], P.mwidth) * ca for i in range(nm)]).astype(dt)
    t0 = time.perf_counter()
    dphi_s, itq, _ = O.solve(m.rowptr, m.colidx, val, qvec[qs], meth, "ICH", tol, 0, threads)
    aphi_s, itm, _ = O.solve(m.rowptr, m.colidx, val, mvec[ms], meth, "ICH", tol, 0, threads)
    t_solve = time.perf_counter() - t0
    nsolved = len(qs) + len(ms)
    # Jacobian sample: nq_jac_sample sources x the sampled detectors (threads share the links)
    jq = min(nq_jac_sample, len(qs))
    links_ofs = np.arange(jq + 1, dtype=np.int32) * len(ms)
    links_m = np.tile(np.arange(len(ms), dtype=np.int32), jq)
    proj = O.project(dphi_s[:jq], mvec[ms], links_ofs, links_m, logscale=False)
    t0 = time.perf_counter()
    O.jacobian(m, dphi_s[:jq], aphi_s, proj, links_ofs, links_m, True, threads)
    t_jac = time.perf_counter() - t0
    pairs_sample = jq * len(ms)
    t_full = t_reset + t_solve * (nq + nm) / nsolved + t_jac * (nq * nm) / pairs_sample
    sample = (f"full assembly+IC(0) factor, {len(qs)}+{len(ms)} of {nq}+{nm} {meth}+ICH solves, "
              f"Jacobian rows of {pairs_sample} of {nq * nm} links; extrapolated linearly to one request")
    return dict(t_request=t_full, t_reset=t_reset, t_solve_sample=t_solve, t_jac_sample=t_jac,
                its_per_src=float(np.mean(np.concatenate([itq, itm]))), threads=threads, sample=sample)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    P = problem(args.config)
    nsolves = P.qm.nQ + P.qm.nM
    times = []
    info = None
    for s in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        # one solve per host thread in each leg, so the sample keeps every core busy
        info = cpu_request_time(P, tol=args.tol)
        if s >= args.warmup:
            times.append(info["t_request"])
    t = float(np.mean(times))
    val = nsolves / t
    line = {"metric": metric_of(args.config), "value": val, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "complex-f64" if P.complex else "f64",
            "data": "synthetic (seeded mesh, optodes, inclusions)",
            "config": {"workload": workload_of(P, args.config, len(P.elems), args.tol, "fp64"),
                       "parallelism": "threads over sources (host)"},
            "impl": "reference",
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": info["threads"], "kind": "port",
                             "sample": info["sample"]},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gpu(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from toastpp_gb300 import build as B
    B.build()
    from toastpp_gb300 import capi

    P = problem(args.config)
    n, nq, nm = P.n, P.qm.nQ, P.qm.nM
    nqm = P.qm.nQM
    cplx = P.complex
    meth = method_of(P)
    cdt = np.complex128 if cplx else np.float64
    gm = capi.Mesh(P.coords, P.elems)
    cm, ck, ca = capi.optical_coefficients(P.mua, P.mus, P.nref)
    omega = capi.omega_of(P.freq_mhz)
    qvec = gm.qvec_gaussian(P.qm.Q, P.qwidth).astype(cdt)
    mvec = (gm.qvec_gaussian(P.qm.M, P.mwidth) * ca[None, :]).astype(cdt)
    vmul = 2 if cplx else 1
    jcols = 2 * n if cplx else n
    links = capi.Links(P.qm.link_ofs, P.qm.link_m)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)   # the library launches on this stream
    torch.cuda.set_stream(stream)
    j_fp32 = {"fp64": 0, "fp32": 1, "fp32acc": 2}[args.jac]

    def dtensor(a):
        a = np.ascontiguousarray(a)
        if np.iscomplexobj(a):
            a = a.view(np.float64)
        return torch.from_numpy(a.copy()).to(dev)

    d_cm, d_ck, d_ca = dtensor(cm), dtensor(ck), dtensor(ca)
    d_q, d_m = dtensor(qvec), dtensor(mvec)
    d_proj = torch.empty(vmul * nqm, dtype=torch.float64, device=dev)
    d_lproj = torch.empty(vmul * nqm, dtype=torch.float64, device=dev)
    d_J = torch.empty((2 * nqm, jcols), dtype=torch.float32 if j_fp32 else torch.float64, device=dev)
    torch.cuda.synchronize()

    s = capi.FwdSolver(gm, meth, args.tol, "ICH", cplx, precision=args.precision)
    s.set_stream(stream.cuda_stream)
    if args.precision == "mixed":
        s.set_refinement(args.inner_tol, 12, args.inner_order)
        s.set_reliable_updates({"restart": 0, "bicgstab": 1, "cocg": 2}[args.inner])
        s.set_backward_error(args.cw_tol)
    res = (capi.TgResult * (nq + nm))()

    def step():
        s.forward_path_raw(d_cm, d_ck, d_ca, omega, nq, d_q, nm, d_m, links, None, None, d_proj, d_lproj, d_J,
                           j_fp32, capi.MEM_DEVICE, res)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    # timed region: device-resident inputs, no profiling events inside; the
    # Jacobian written every step (3 GB at the default size) flushes L2
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    l0 = capi.launch_count()
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(args.steps):
            evs[i][0].record(stream)
            step()
            evs[i][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    launches = capi.launch_count() - l0
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = float(np.sum(step_ms))
    if ws > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    its = [r.it_count for r in res]
    # per-class device time from separate profiled steps (CUDA events around
    # each launch class, on the library's stream), outside the timed region
    psteps = max(1, min(2, args.steps))
    s.profile((1 << capi.PROF_SPMM) | (1 << capi.PROF_SWEEP) | (1 << capi.PROF_JAC) | (1 << capi.PROF_ASM)
              | (1 << capi.PROF_PROJ))
    for _ in range(psteps):
        step()
    torch.cuda.synchronize()
    prof = {c: s.profile_read(c) for c in (capi.PROF_SPMM, capi.PROF_SWEEP, capi.PROF_JAC, capi.PROF_ASM,
                                           capi.PROF_PROJ)}
    s.profile(0)
    nsolves = nq + nm
    value = ws * nsolves * args.steps / (total_ms / 1e3)

    # roofline of the dominant class (algorithmic bytes per launch / event-timed duration)
    nnz = gm.nnz
    k_f = nq + nm          # forward and adjoint sources share one batch
    nnz_l = (nnz - n) // 2
    names = {capi.PROF_SPMM: f"SpMM (autotuned spmm_halo/vec/wide kernel, k={nq + nm})",
             capi.PROF_SWEEP: "IC(0) apply: the level kernels of both sweeps (ic_level_ell) in one graph",
             capi.PROF_JAC: ("jacobian_kernel (FP32)" if j_fp32 == 1 else
                             ("jacobian_oz_kernel (tensor cores: exact bf16 digit products, %s J)" if cplx else
                              "jacobian_ff_kernel (float-float arithmetic, %s J)") % ("FP32" if j_fp32 else "FP64")),
             capi.PROF_ASM: "assembly + IC(0) factor", capi.PROF_PROJ: "project_kernel"}
    dom = max(prof, key=lambda c: prof[c][0])
    vb = (8 if args.precision == "mixed" else 16) // (1 if cplx else 2)
    jb = 4 if j_fp32 else 8
    tc = dom == capi.PROF_JAC and cplx and j_fp32 != 1  # the tensor-core Jacobian
    if tc:
        # the digit products: per node a real (2nq x 2deg) x (2deg x 2nm)
        # product per digit pair, 28 pairs (7 digits per operand); the sum of
        # the node degrees is the number of CSR entries
        alg_flops = 28 * 16.0 * nq * nm * nnz
        alg_bytes = 2 * nqm * jcols * jb + (nq + nm) * n * vb + (n + 1 + nnz) * 4
    elif dom == capi.PROF_JAC:
        # J write + fields read once + CSR pattern (per launch)
        alg_bytes = 2 * nqm * jcols * jb + (nq + nm) * n * vb + (n + 1 + nnz) * 4
    elif dom == capi.PROF_SPMM:
        alg_bytes = nnz * (vb + 4) + 4 * (n + 1) + 2 * n * k_f * vb
    elif dom == capi.PROF_SWEEP:
        alg_bytes = 2 * (nnz_l * (vb + 4) + 4 * (n + 1)) + n * vb + 4 * n * k_f * vb
    else:
        alg_bytes = None
    dom_ms, dom_cnt = prof[dom]
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    roof = None
    if tc and dom_cnt:
        t_launch = dom_ms / dom_cnt / 1e3
        tpeak = peaks.get("bf16_tflops", 1900.0)
        ach = alg_flops / t_launch / 1e12
        roof = {"bound": "tensor", "kernel": names[dom], "achieved": ach, "peak": tpeak, "unit": "TFLOP/s",
                "frac": ach / tpeak, "peak_source": "measured" if "bf16_tflops" in peaks else "fallback",
                "traffic": None, "algorithmic_flops_per_launch": alg_flops,
                "algorithmic_bytes_per_launch": alg_bytes, "launch_ms": dom_ms / dom_cnt,
                "hbm_view": {"achieved_gbs": alg_bytes / t_launch / 1e9, "frac": alg_bytes / t_launch / 1e9 / peak},
                "note": ("bf16 mma.sync digit products (measured ceiling of that instruction on this GPU: about "
                         "600 TFLOP/s); the float-float digit preparation and the float-float recombination, "
                         "1/y scaling and FP64 rounding of each entry run on the CUDA cores")}
        tr = TRAFFIC.get((args.config, "jacobian_oz"))
        if tr:
            roof["traffic"] = tr[0]
            roof["traffic_source"] = tr[1]
    elif alg_bytes and dom_cnt:
        ach = alg_bytes / (dom_ms / dom_cnt / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": names[dom], "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": ach / peak, "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                "traffic": None, "algorithmic_bytes_per_launch": alg_bytes,
                "launch_ms": dom_ms / dom_cnt}
        tr = TRAFFIC.get((args.config, dom == capi.PROF_JAC and j_fp32 == 0 and "jacobian_ff"
                          or dom == capi.PROF_SWEEP and "ic_level_ell" or None))
        if tr:
            # ncu dram__bytes_read.sum + dram__bytes_write.sum per launch,
            # from a capture of a smaller case scaled by the units processed
            roof["traffic"] = tr[0]
            roof["traffic_source"] = tr[1]
        if dom == capi.PROF_JAC and j_fp32 != 1:
            roof["note"] = ("the float-float Jacobian is bound by FP32 issue (packed f32x2 pipe), not by HBM: "
                            "its J write is the only large traffic")
    shares = {names[c]: {"ms_per_step": prof[c][0] / psteps, "launches_or_scopes": prof[c][1] // psteps}
              for c in prof}

    # ---- grid-basis Jacobian (pixel raster, basis = grid) and, with
    # --element, the element-basis Jacobian on this request's fields,
    # device-resident, each timed alone with CUDA events (mean of reps calls
    # after 3 untimed ones)
    def event_ms(fn, reps=5):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, b in ev:
            a.record(stream)
            fn()
            b.record(stream)
        torch.cuda.synchronize()
        return float(np.mean([a.elapsed_time(b) for a, b in ev]))

    grid = element = None
    # one more request with its fields kept: the inputs of the grid / element
    # Jacobian legs and of the comparison with the oracle
    d_dphi = torch.empty((nq, n * vmul), dtype=torch.float64, device=dev)
    d_aphi = torch.empty((nm, n * vmul), dtype=torch.float64, device=dev)
    s.forward_path_raw(d_cm, d_ck, d_ca, omega, nq, d_q, nm, d_m, links, d_dphi, d_aphi, d_proj, d_lproj, d_J,
                       j_fp32, capi.MEM_DEVICE, res)
    torch.cuda.synchronize()
    fields = {"dphi": d_dphi, "aphi": d_aphi, "proj": d_proj.clone(), "lproj": d_lproj.clone(), "J": d_J}
    if args.grid > 0:
        rast = capi.Raster(gm, [args.grid] * P.dim)
        gcols = (2 if cplx else 1) * rast.slen
        # the grid and element legs time FP32 Jacobians (their own bases' kernels)
        d_Jg = torch.empty((2 * nqm, gcols), dtype=torch.float32, device=dev)

        def gstep():
            s.jacobian_grid_raw(rast, nq, d_dphi, nm, d_aphi, d_proj, links, capi.DATA_LOG, d_Jg, True,
                                capi.MEM_DEVICE)

        g_ms = event_ms(gstep)
        jb = d_Jg.numel() * d_Jg.element_size()
        # field planes read once per source / detector (value + dim gradients)
        pb = (nq + nm) * (1 + P.dim) * rast.slen * 8 // (1 if cplx else 2)
        peak = peaks.get("hbm_gbs", 6800.0)
        grid = {"raster": [args.grid] * P.dim, "solution_points": rast.slen, "ms_per_jacobian": g_ms,
                "jacobians_per_s": 1e3 / g_ms, "J_bytes": jb,
                "roofline": {"bound": "hbm", "achieved": (jb + pb) / (g_ms / 1e3) / 1e9, "peak": peak,
                             "unit": "GB/s", "frac": (jb + pb) / (g_ms / 1e3) / 1e9 / peak,
                             "algorithmic_bytes_per_launch": jb + pb},
                "note": "FP32 J; includes the field resampling and gradient launches; inputs on the device"}
        rast.close()
        del d_Jg
    if args.element:
        # element-basis Jacobian (one column per element and component) on the same fields
        ecols = (2 if cplx else 1) * gm.ne
        d_Je = torch.empty((2 * nqm, ecols), dtype=torch.float32, device=dev)
        e_ms = event_ms(lambda: s.jacobian_el_raw(nq, d_dphi, nm, d_aphi, d_proj, links, capi.DATA_LOG, d_Je,
                                                  True, capi.MEM_DEVICE))
        jb = d_Je.numel() * d_Je.element_size()
        fb = (nq + nm) * n * vmul * 8  # the FP64 fields, read once
        element = {"elements": gm.ne, "ms_per_jacobian": e_ms, "jacobians_per_s": 1e3 / e_ms, "J_bytes": jb,
                   "roofline": {"bound": "hbm", "achieved": (jb + fb) / (e_ms / 1e3) / 1e9, "peak": peak,
                                "unit": "GB/s", "frac": (jb + fb) / (e_ms / 1e3) / 1e9 / peak,
                                "algorithmic_bytes_per_launch": jb + fb},
                   "note": "includes the FP32 casts of the fields; inputs on the device"}
        del d_Je

    # ---- e2e through the C ABI with host buffers (pinned), copies inside the timed region
    e2e = None
    j_bytes = 2 * nqm * jcols * (4 if j_fp32 else 8)
    if (rank == 0 or ws > 1) and not args.no_e2e and j_bytes <= 16e9:
        h_cm, h_ck, h_ca = (torch.from_numpy(np.ascontiguousarray(x)).pin_memory() for x in (cm, ck, ca))
        h_q = torch.from_numpy(np.ascontiguousarray(qvec).view(np.float64).copy()).pin_memory()
        h_m = torch.from_numpy(np.ascontiguousarray(mvec).view(np.float64).copy()).pin_memory()
        h_proj = torch.empty(vmul * nqm, dtype=torch.float64).pin_memory()
        h_lproj = torch.empty(vmul * nqm, dtype=torch.float64).pin_memory()
        h_J = torch.empty((2 * nqm, jcols), dtype=torch.float32 if j_fp32 else torch.float64).pin_memory()
        ksteps = max(1, min(args.steps, 3))
        s.forward_path_raw(h_cm, h_ck, h_ca, omega, nq, h_q, nm, h_m, links, None, None, h_proj, h_lproj, h_J,
                           j_fp32, capi.MEM_HOST)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(ksteps):
            s.forward_path_raw(h_cm, h_ck, h_ca, omega, nq, h_q, nm, h_m, links, None, None, h_proj, h_lproj, h_J,
                               j_fp32, capi.MEM_HOST)
        torch.cuda.synchronize()
        te = time.perf_counter() - t0
        h2d = 3 * n * 8 + (nq + nm) * n * 8 * vmul + (nq + 1 + nqm) * 4
        d2h = 2 * nqm * 8 * vmul + h_J.numel() * h_J.element_size()
        serial = ws * nsolves * ksteps / te
        e2e = {"value": serial, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "steps": ksteps, "api": "tg_forward_path, one request at a time, page-locked host buffers"}
    # the server's solvers take the library's default refinement settings
    defaults = args.precision == "fp64" or (args.inner_tol == 1e-4 and args.inner_order == 1 and args.inner == "cocg"
                                            and args.cw_tol == 1e-10)
    if e2e is not None and defaults:
        # the same requests through the request server: request i + 1 solves
        # while request i's Jacobian streams to host memory (deferred output)
        pdt = np.complex128 if cplx else np.float64
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
        p_cm, p_ck, p_ca, p_q, p_m = pin(cm), pin(ck), pin(ca), pin(qvec.astype(pdt)), pin(mvec.astype(pdt))
        outs = [(pin(np.zeros(nqm, pdt)), pin(np.zeros(nqm, pdt)), h_J.numpy() if b == 0 else
                 torch.empty(tuple(h_J.shape), dtype=h_J.dtype).pin_memory().numpy()) for b in range(2)]
        srv = capi.Server(slots=args.e2e_slots, hbm_budget_gb=200.0)

        def request(b):
            return capi.Request(gm, p_cm, p_ck, p_ca, omega, p_q, p_m, links, solver=meth, precon="ICH",
                                tol=args.tol, precision=args.precision, want_jac=True, j_fp32=j_fp32, outputs=outs[b])

        for t in [srv.submit(request(b)) for b in range(2)]:
            srv.wait(t)
        psteps_e2e = max(10, 2 * ksteps)
        t0 = time.perf_counter()
        tickets = [srv.submit(request(i % 2)) for i in range(psteps_e2e)]
        done = [srv.wait(t) for t in tickets]
        tp = time.perf_counter() - t0
        srv.close()
        bad = sum(1 for rq in done for r in rq.results if r[1] != 0)
        e2e = {"value": ws * nsolves * psteps_e2e / tp, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "steps": psteps_e2e,
               "api": f"tg_submit / tg_wait, request server with {args.e2e_slots} slot(s), page-locked host buffers",
               "unconverged_sources": bad,
               "serial": {"value": serial, "steps": ksteps,
                          "api": "tg_forward_path, one request at a time, page-locked host buffers"}}

    # ---- two requests on the device at once (two solvers, two streams, two
    # host threads, inputs resident): what the request server's slots do
    concurrent = None
    if not args.no_concurrent and j_bytes <= 16e9:
        concurrent = concurrent_leg(args, gm, meth, cplx, omega, nq, nm, (d_cm, d_ck, d_ca, d_q, d_m), links, dev,
                                    j_fp32, (vmul * nqm, (2 * nqm, jcols)), nsolves, ws)

    line = None
    if rank == 0:
        # ---- FP64 comparison legs (same request, plain FP64)
        compare = {}
        if not args.no_compare:
            compare = compare_legs(args, P, gm, s, stream, dev, links, (d_cm, d_ck, d_ca), omega, (d_q, d_m),
                                   (cm, ck, ca, qvec, mvec), fields, value, res_kind=meth)
        cpu = None
        if not args.no_cpu:
            info = cpu_request_time(P, tol=args.tol)
            cpu = {"value": nsolves / info["t_request"], "unit": UNIT, "cores": info["threads"], "kind": "port",
                   "sample": info["sample"], "its_per_src": info["its_per_src"]}
        serving_leg = None
        if not args.no_serving and ws == 1:
            torch.cuda.synchronize()
            wl, sv = serving_summary(args, 12, 10.0, args.slots)
            serving_leg = {"workload": wl, "slots": args.slots,
                           "mixed": {k: sv["mixed"][k] for k in ("p50_ms", "p99_ms", "solves_per_s", "requests")},
                           "fp64": {k: sv["fp64"][k] for k in ("p50_ms", "p99_ms", "solves_per_s", "requests")},
                           "saturated_solves_per_s": {"mixed": sv["mixed_saturated"]["solves_per_s"],
                                                      "fp64": sv["fp64_saturated"]["solves_per_s"]},
                           "per_mesh_p50_ms_mixed": sv["mixed"]["per_mesh_p50_ms"]}
        clocks = clk.summary()
        line = {
            "metric": metric_of(args.config), "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": ((("complex-f32" if cplx else "f32") + " inner / " + ("complex-f64" if cplx else "f64") +
                       " refinement") if args.precision == "mixed" else ("complex-f64" if cplx else "f64")),
            "data": "synthetic (seeded mesh, optodes, inclusions)",
            "config": {"workload": workload_of(P, args.config, gm.ne, args.tol, args.precision,
                                               f" (inner FP32 tol {args.inner_tol}, componentwise backward error "
                                               f"<= {args.cw_tol}, J {args.jac})"
                                               if args.precision == "mixed" else ""),
                       "parallelism": f"replicas x{ws} (one request per GPU)",
                       "l2": f"each step writes the {j_bytes / 1e9:.2f} GB Jacobian"
                             + (", larger than L2" if j_bytes > 130e6 else ", smaller than L2: L2-resident case")},
            "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99))},
            "jacobians_per_s": ws * args.steps / (total_ms / 1e3),
            "iterations_per_source": float(np.mean(its)),
            "unconverged_sources": int(sum(1 for r in res if r.status != 0)),
            "ic_applies_per_request": prof[capi.PROF_SWEEP][1] / psteps,
            "roofline": roof, "kernel_time_per_step": shares,
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches), "grid_jacobian": grid,
            "element_jacobian": element,
            "clocks": clocks, "wall_s": wall, "compare": compare, "serving": serving_leg,
            "concurrent_requests": concurrent,
            "spmm_autotuner": capi.tuner_log().strip().splitlines(),
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return 0


def concurrent_leg(args, gm, meth, cplx, omega, nq, nm, d_in, links, dev, j_fp32, shapes, nsolves, ws, nreq=2,
                   rounds=6):
    """nreq requests at once: one solver, stream and host thread each, the
    same device-resident inputs; wall time of `rounds` requests per thread
    after one untimed round (the GIL is released inside the library calls)."""
    import torch
    from toastpp_gb300 import capi
    d_cm, d_ck, d_ca, d_q, d_m = d_in
    (np_lin, jshape) = shapes
    work = []
    for _ in range(nreq):
        st = torch.cuda.Stream(device=dev)
        s = capi.FwdSolver(gm, meth, args.tol, "ICH", cplx, precision=args.precision)
        s.set_stream(st.cuda_stream)
        if args.precision == "mixed":
            s.set_refinement(args.inner_tol, 12, args.inner_order)
            s.set_reliable_updates({"restart": 0, "bicgstab": 1, "cocg": 2}[args.inner])
            s.set_backward_error(args.cw_tol)
        out = (torch.empty(np_lin, dtype=torch.float64, device=dev), torch.empty(np_lin, dtype=torch.float64, device=dev),
               torch.empty(jshape, dtype=torch.float32 if j_fp32 else torch.float64, device=dev))
        work.append((s, out))

    def run(i, reps):
        s, (pr, lp, J) = work[i]
        for _ in range(reps):
            s.forward_path_raw(d_cm, d_ck, d_ca, omega, nq, d_q, nm, d_m, links, None, None, pr, lp, J, j_fp32,
                               capi.MEM_DEVICE)

    def timed(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ths = [threading.Thread(target=run, args=(i, reps)) for i in range(nreq)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    timed(1)
    dt = timed(rounds)
    for s, _ in work:
        s.close()
    return {"value": ws * nreq * rounds * nsolves / dt, "unit": UNIT, "requests_at_once": nreq,
            "ms_per_round": dt * 1e3 / rounds, "rounds": rounds,
            "api": "tg_forward_path on two solvers and streams from two host threads, inputs on the device"}


def compare_legs(args, P, gm, s, stream, dev, links, d_par, omega, d_src, h_src, fields, value, res_kind):
    """Error of the measured request against the FP64 oracle, and the plain
    FP64 GPU baselines, all outside the timed region:

    - vs_oracle: the oracle's exact FP64 solve of the same request (the
      direct factorisation in a nested-dissection ordering, every source and
      detector), its projections, and its Jacobian rows for a sample of links;
    - fp64_batched: the same request through the plain FP64 path (the
      reference's recursion, all right-hand sides in one block) and that
      path's own error against the oracle;
    - fp64_per_source_solve: the plain FP64 solve one right-hand side per
      call, device-resident, timed with CUDA events over 16 sources;
    - jacobian_fp32_variant: the same request with an FP32 Jacobian.
    """
    import torch
    from toastpp_gb300 import capi
    from oracle import oracle as O
    cm, ck, ca, qvec, mvec = h_src
    d_cm, d_ck, d_ca = d_par
    d_q, d_m = d_src
    n, nq, nm, nqm = P.n, P.qm.nQ, P.qm.nM, P.qm.nQM
    cplx = P.complex
    cdt = np.complex128 if cplx else np.float64
    nsolves = nq + nm
    out = {}
    # ---- the oracle's exact FP64 solve
    t0 = time.perf_counter()
    om = O.Mesh(P.coords, P.elems)
    ocm, ock, oca = O.optical_coefficients(P.mua, P.mus, P.nref)
    val = om.assemble(ocm, ock, oca, P.freq_mhz * 2 * np.pi * 1e-6, cplx)
    oq = np.stack([om.qvec_gaussian(q, P.qwidth) for q in P.qm.Q]).astype(cdt)
    omv = np.stack([om.qvec_gaussian(m, P.mwidth) * oca for m in P.qm.M]).astype(cdt)
    th = os.cpu_count() or 1
    if n <= 60000:
        # every source and detector: the direct factorisation
        D = O.Direct(om.rowptr, om.colidx, val, "nd", om.coords)
        qs, ms = np.arange(nq), np.arange(nm)
        Xq = D.solve(oq, th)
        Xm = D.solve(omv, th)
        how = "direct factorisation (nested-dissection order), every source and detector"
    else:
        # a sample: BiCGSTAB + ICH restarted from the true FP64 residual until
        # the componentwise backward error is 1e-12 (too large to factor)
        qs, ms = np.arange(min(8, nq)), np.arange(min(8, nm))
        X, _ = O.solve_refined(om.rowptr, om.colidx, val, np.concatenate([oq[qs], omv[ms]]), nthreads=th)
        Xq, Xm = X[:len(qs)], X[len(qs):]
        how = (f"FP64 BiCGSTAB+ICH refined to componentwise backward error 1e-12, sources {len(qs)} and "
               f"detectors {len(ms)} of {nq} + {nm}")
    # links of the sampled sources (all detectors), and for the Jacobian the
    # links of the first sampled sources to the sampled detectors
    ofs_all = np.asarray(P.qm.link_ofs, np.int32)
    lm_all = np.asarray(P.qm.link_m, np.int32)
    lsel = np.concatenate([np.arange(ofs_all[q], ofs_all[q + 1]) for q in qs])
    pofs = np.concatenate([[0], np.cumsum([ofs_all[q + 1] - ofs_all[q] for q in qs])]).astype(np.int32)
    pref = O.project(Xq, omv, pofs, lm_all[lsel], logscale=False)
    lref = O.project(Xq, omv, pofs, lm_all[lsel], logscale=True)
    jq = min(4, len(qs))
    mpos = {int(m): i for i, m in enumerate(ms)}
    jl, jm = [], []
    jofs = [0]
    for q in qs[:jq]:
        for l in range(ofs_all[q], ofs_all[q + 1]):
            if int(lm_all[l]) in mpos:
                jl.append(l)
                jm.append(mpos[int(lm_all[l])])
        jofs.append(len(jl))
    jl = np.array(jl)
    ylin = pref[[int(np.nonzero(lsel == l)[0][0]) for l in jl]]
    Jref = O.jacobian(om, Xq[:jq], Xm, ylin, np.array(jofs, np.int32), np.array(jm, np.int32), True, th)
    t_oracle = time.perf_counter() - t0

    def errors(dphi, aphi, proj, lproj, J):
        e = {}
        fq = dphi.cpu().numpy().view(cdt)[qs] if dphi is not None else None
        if fq is not None:
            fm = aphi.cpu().numpy().view(cdt)[ms]
            e["fields_l2"] = float(np.sqrt((np.linalg.norm(fq - Xq) ** 2 + np.linalg.norm(fm - Xm) ** 2) /
                                           (np.linalg.norm(Xq) ** 2 + np.linalg.norm(Xm) ** 2)))
        pg = proj.cpu().numpy().view(cdt)[lsel]
        lg = lproj.cpu().numpy().view(cdt)[lsel]
        e["boundary_data_max_rel_linear"] = float(np.max(np.abs(pg - pref) / np.abs(pref)))
        e["boundary_data_l2_rel_linear"] = float(np.linalg.norm(pg - pref) / np.linalg.norm(pref))
        ok = np.isfinite(lg) & np.isfinite(lref)
        e["boundary_data_max_abs_log"] = float(np.max(np.abs(lg - lref)[ok]))
        if J is not None:
            nl = len(jl)
            rows = np.concatenate([jl, nqm + jl])
            Jg = J[torch.as_tensor(rows, device=J.device)].double().cpu().numpy()
            Jr = Jref.reshape(2 * nl, -1)
            e["jacobian_l2_rel_sampled_rows"] = float(np.linalg.norm(Jg - Jr) / np.linalg.norm(Jr))
        return e

    f = fields
    out["vs_oracle"] = {"oracle": f"exact FP64 solve of the same request ({how}), projections of "
                                  f"{len(lsel)} links, Jacobian rows of {len(jl)} links",
                        "oracle_s": t_oracle, **errors(f["dphi"], f["aphi"], f["proj"], f["lproj"], f["J"])}
    # ---- plain FP64 path, batched (the reference's recursion)
    s64 = capi.FwdSolver(gm, res_kind, args.tol, "ICH", cplx, precision="fp64")
    s64.set_stream(stream.cuda_stream)
    jcols = 2 * n if cplx else n
    # the FP64 path's Jacobian only where it is modest (16 GB)
    d_J64 = (torch.empty((2 * nqm, jcols), dtype=torch.float64, device=dev) if 2 * nqm * jcols * 8 <= 16e9
             else None)
    p64 = torch.empty_like(f["proj"])
    lp64 = torch.empty_like(f["lproj"])
    s64.forward_path_raw(d_cm, d_ck, d_ca, omega, nq, d_q, nm, d_m, links, None, None, p64, lp64, d_J64, 0,
                         capi.MEM_DEVICE)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    s64.forward_path_raw(d_cm, d_ck, d_ca, omega, nq, d_q, nm, d_m, links, None, None, p64, lp64, d_J64, 0,
                         capi.MEM_DEVICE)
    b.record(stream)
    torch.cuda.synchronize()
    t64 = a.elapsed_time(b) / 1e3
    out["fp64_batched"] = {"value": nsolves / t64, "unit": UNIT, "ms_per_request": t64 * 1e3,
                           "tol": args.tol, "vs_oracle": errors(None, None, p64, lp64, d_J64)}
    del d_J64, s64
    # ---- plain FP64, one right-hand side per call, device-resident
    s1 = capi.FwdSolver(gm, res_kind, args.tol, "ICH", cplx, precision="fp64")
    s1.set_stream(stream.cuda_stream)
    s1.reset(d_cm, d_ck, d_ca, omega, capi.MEM_DEVICE)
    ns = min(16, nq)
    vm = 2 if cplx else 1
    d_phi1 = torch.zeros((ns, n * vm), dtype=torch.float64, device=dev)
    r1 = (capi.TgResult * 1)()
    s1.calc_fields_raw(1, d_q[0], d_phi1[0], capi.MEM_DEVICE, r1)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(ns)]
    its1 = []
    for i in range(ns):
        ev[i][0].record(stream)
        s1.calc_fields_raw(1, d_q[i], d_phi1[i], capi.MEM_DEVICE, r1)
        ev[i][1].record(stream)
        its1.append(r1[0].it_count)
    torch.cuda.synchronize()
    tps = float(np.mean([x.elapsed_time(y) for x, y in ev])) / 1e3
    out["fp64_per_source_solve"] = {"value": 1.0 / tps, "unit": "source-solves/s (solve only)",
                                    "ms_per_solve": tps * 1e3, "iterations_per_source": float(np.mean(its1)),
                                    "sample": f"{ns} single-RHS solves, device-resident, CUDA events"}
    out["speedup_vs_fp64_per_source_solve"] = value / (1.0 / tps)
    del s1, d_phi1
    # ---- the same request with an FP32 Jacobian (FP32 products of the refined fields)
    if args.precision == "mixed" and args.jac == "fp64" and 2 * nqm * jcols * 4 <= 32e9:
        d_J32 = torch.empty((2 * nqm, jcols), dtype=torch.float32, device=dev)
        p32 = torch.empty_like(f["proj"])
        lp32 = torch.empty_like(f["lproj"])
        r32 = (capi.TgResult * nsolves)()
        for _ in range(2):
            s.forward_path_raw(d_cm, d_ck, d_ca, omega, nq, d_q, nm, d_m, links, None, None, p32, lp32, d_J32, 1,
                               capi.MEM_DEVICE, r32)
        torch.cuda.synchronize()
        k32 = 3
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k32)]
        for x, y in ev:
            x.record(stream)
            s.forward_path_raw(d_cm, d_ck, d_ca, omega, nq, d_q, nm, d_m, links, None, None, p32, lp32, d_J32, 1,
                               capi.MEM_DEVICE, r32)
            y.record(stream)
        torch.cuda.synchronize()
        t32 = float(np.mean([x.elapsed_time(y) for x, y in ev])) / 1e3
        e32 = errors(None, None, p32, lp32, d_J32)
        out["jacobian_fp32_variant"] = {"value": nsolves / t32, "unit": UNIT, "ms_per_request": t32 * 1e3,
                                        "jacobian_l2_rel_sampled_rows": e32["jacobian_l2_rel_sampled_rows"]}
        del d_J32
    return out


def serving_summary(args, requests, rate, slots):
    """The serving stream (Poisson arrivals over the 2D 3.3k / 2D 13k / 3D 30k /
    3D 250k meshes, 8-128 sources (at most --src-max-large on the box), CW or
    100 MHz, fresh parameters per request) through the request server, mixed
    precision and plain FP64: p50 / p99 latency and source-solves/s at the
    given arrival rate, and the same requests all arriving at once."""
    from toastpp_gb300 import serving
    ms = serving.MeshSet()
    out = {}
    for prec in ("mixed", "fp64"):
        spec = serving.StreamSpec(requests=requests, rate_hz=rate, seed=1, precision=prec, tol=1e-10,
                                  src_max_large=args.src_max_large)
        # one pass over a short stream first, so that every solver and graph is resident
        warm = serving.make_requests(ms, serving.StreamSpec(requests=min(8, requests), rate_hz=1e6, seed=2,
                                                            precision=prec, tol=1e-10,
                                                            src_max_large=args.src_max_large))
        serving.run_stream(warm, slots=slots)
        del warm
        reqs = serving.make_requests(ms, spec)
        done, st, wall = serving.run_stream(reqs, slots=slots)
        out[prec] = serving.summarize(done, st, wall)
        del reqs, done
        sat = serving.make_requests(ms, serving.StreamSpec(requests=requests, rate_hz=1e6, seed=1, precision=prec,
                                                           tol=1e-10, src_max_large=args.src_max_large))
        done, st, wall = serving.run_stream(sat, slots=slots)
        out[prec + "_saturated"] = serving.summarize(done, st, wall)
        del sat, done
    workload = (f"Poisson arrivals {rate}/s, meshes 2D 3.3k/2D 13k/3D 30k/3D 250k (0.4/0.3/0.2/0.1), 8-128 sources "
                f"(<= {args.src_max_large} on the 250k box: 16 GB FP32 Jacobian per request at 64), CW or 100 MHz, "
                "forward + projections + nodal FP32 Jacobian per request, tol 1e-10")
    return workload, out


def run_serving(args):
    """The serving stream alone, as its own JSON line."""
    import torch
    torch.cuda.set_device(0)
    from toastpp_gb300 import build as B
    B.build()
    workload, out = serving_summary(args, args.requests, args.rate, args.slots)
    m = out["mixed"]
    line = {"metric": "serving stream: source-solves/s with p50/p99 request latency", "value": m["solves_per_s"],
            "unit": "source-solves/s", "n_gpus": 1, "steps": args.requests, "warmup": 8, "higher_is_better": True,
            "dtype": "complex-f32 inner / complex-f64 refinement (mixed); complex-f64 (fp64 leg)",
            "data": "synthetic (seeded meshes, optodes, parameter fields, arrivals)",
            "config": {"workload": workload, "slots": args.slots},
            "latency_ms": {"p50": m["p50_ms"], "p99": m["p99_ms"]}, "mixed": m, "fp64": out["fp64"],
            "saturated": {"mixed": out["mixed_saturated"], "fp64": out["fp64_saturated"]}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.serving:
        return run_serving(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
