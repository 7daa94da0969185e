"""Benchmark: chiqw seconds per q-point (all frequencies) on one GB300.

Workload ``chiqw_8x8x8k_200b`` (seeded synthetic, no dataset): fcc cell
a = 15.84 bohr, 8x8x8 Gamma-centred k mesh (512 q), 200 bands (8 occupied,
1536 band pairs), 20 Ry wave-function cutoff (~1514 plane waves), FFT box 36^3,
dielectric cutoff 11 Ry (~600 G), 20 frequencies (10 real 0-30 eV, 10
imaginary on a Gauss-Legendre grid over 0-30 eV), band-cRPA window 9-11.

A step is one q point: rp_chi0_q (tetrahedron weights, pair densities,
contraction) + rp_epsinv_q (eps build and inversion: FP32 Gauss-Jordan plus
one float-pair Newton step, the FP64 Gauss-Jordan as fallback).  `value` is
the device time per q point of the split-precision (FP16x3) path with every
input resident in HBM; `e2e` is the same q points again through the C ABI
with host output buffers (chi and eps^-1 copied back every step).  Inputs
(38 GB of real-space wave functions, 3.8 GB of pair densities per q) are
larger than L2, so no flush is needed.  The plain FP64 GPU path and the chi
and eps^-1 errors of the fast path are measured on a 96-pair sample of the
first timed q and scaled linearly in the pair count (every stage but the eps
inversion is linear in it).  The CPU baseline is the C restatement (oracle)
on the host cores on a bounded sample (pairs and k points), scaled the same
way.  The default line also carries the ragged-batch leg (`ragged`).

--impl reference runs that CPU restatement as the reference arm on the GPU
arm's timed q points: the reference (Fortran + MPI + MKL) cannot be built
here (no Fortran compiler).
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

AU = 27.21151
WORKLOAD = "chiqw_8x8x8k_200b"
METRIC = "chiqw s/q-point (all w) vs plain FP64 GPU at chi rel err<=1e-6; % roofline"


def make_spec(case="full"):
    from respackdev_gb300 import synth
    # small: the same cell, cutoffs, FFT box and frequencies on a 4x4x4 mesh with
    # 100 bands -- the kernels of the full workload at a size an ncu capture can hold
    return synth.CASES["headline_small" if case == "small" else "headline"]


def frequencies():
    re = np.linspace(0.0, 30.0, 10)
    x, _ = np.polynomial.legendre.leggauss(10)
    im = 15.0 * (x + 1.0)
    return np.concatenate([re, 1j * im]) / AU


RUN_PARAMS = dict(ecut_for_eps=11.0, green_func_delt=0.2721, flg_crpa=1)
FFT_BOX = (36, 36, 36)


def prepare(root, case="full"):
    from respackdev_gb300 import synth
    t = time.time()
    synth.make_case(root, make_spec(case))
    return time.time() - t


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("bf16_tflops_sustained"), d.get("bf16_tflops"), d.get("hbm_gbs"), "measured"
    return 1700.0, 1900.0, 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per tensor-core contraction launch from the committed ncu summary, if any."""
    p = os.path.join(HERE, "profiles", "tc_gram_kernel_chiqw.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch_scaled:"):
            try:
                return float(line.split(":", 1)[1])
            except ValueError:
                return None
    return None


def cpu_baseline(root, nthreads, npair_sample, em, iq, max_k=0):
    """The C restatement on host cores, one q point on a bounded sample: the
    first npair_sample band pairs, and with max_k > 0 their pair densities and
    contraction over the first max_k k points only.  The time is scaled
    linearly to all pairs and all k (the per-pair tetrahedron weights, under
    0.5 % of a pair's time, always run over the whole mesh)."""
    from oracle import oracle as orc
    orc.build()
    shutil.rmtree(os.path.join(root, "dir-eps"), ignore_errors=True)
    p = orc.make_params(em=em, nthreads=nthreads, max_pairs=npair_sample, calc_num_k=[iq], fft_box=FFT_BOX,
                        write_eps=0, max_k=max_k, **RUN_PARAMS)
    rep = orc.calc_chiqw(root, p)
    frac = rep.npair_full_last / max(1, rep.npair_last) * rep.ntk / max(1, rep.nk_used_last)
    return rep.seconds_last_q * frac, rep


def num_qirr(root):
    with open(os.path.join(root, "dir-wfn", "dat.sample-k")) as f:
        return int(f.readline().split()[0])


def shard_q(nq_all: int, rank: int, world: int):
    """q points of one rank: every world-th point after Gamma (weak scaling;
    the reference's MPI_num_qcomm q communities, chiqw.F:662-687)."""
    return list(range(2, nq_all + 1))[rank::world]


def step_q_list(nq_all, rank, world, warmup, steps):
    """The q point of every warm-up and timed step of one rank (cycling if needed)."""
    mine = shard_q(nq_all, rank, world)
    need = warmup + steps
    return (mine * (need // max(1, len(mine)) + 1))[:need]


def workload_config(ntk, nbands, npair, ng, nen, box, qs, world):
    """`config` of both arms: the same workload keys and values."""
    return {"workload": WORKLOAD, "ntk": ntk, "nbands": nbands, "npair": npair, "ng": ng, "nen": nen,
            "fft_box": list(box), "q_points": f"{qs[0]}-{qs[-1]}" if qs else "",
            "l2": "inputs larger than L2 (38 GB wave functions, 3.8 GB pair densities per q)",
            "parallelism": f"q-shard x{world}"}


def run_reference(args):
    """The reference arm: the C restatement of chiqw on the host cores, each
    step one timed q point of the GPU arm's list (a bounded sample of it:
    as many band pairs as threads, over a quarter of the k mesh, scaled
    linearly)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    nthreads = os.cpu_count() or 1
    tmp = tempfile.mkdtemp(prefix="rp_bench_ref_")
    try:
        prepare(tmp)
        em = frequencies()
        qs = step_q_list(num_qirr(tmp), 0, world, args.warmup, args.steps)
        ntk = int(np.prod(make_spec().nk))
        for iq in qs[: args.warmup]:
            cpu_baseline(tmp, 1, 1, em, iq, max_k=8)
        vals, ngs = [], []
        rep = None
        t0 = time.time()
        for iq in qs[args.warmup:]:
            v, rep = cpu_baseline(tmp, nthreads, nthreads, em, iq, max_k=max(1, ntk // 4))
            vals.append(v)
            ngs.append(rep.ng_last)
        wall = time.time() - t0
        value = float(np.mean(vals))
        line = {"metric": METRIC, "value": value, "unit": "s/q-point", "impl": "reference",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
                "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": workload_config(rep.ntk, make_spec().nbands, rep.npair_full_last, ngs[0], rep.nen,
                                          rep.fft_box, qs[args.warmup:], world),
                "ng_per_step": ngs,
                "cpu_baseline": {"value": value, "unit": "s/q-point", "cores": nthreads, "kind": "port",
                                 "sample": f"per step one q point of the GPU arm's timed list, {rep.npair_last} of "
                                           f"{rep.npair_full_last} band pairs over {rep.nk_used_last} of {rep.ntk} "
                                           f"k points, scaled linearly (C restatement of chiqw on {nthreads} threads; "
                                           f"the Fortran reference cannot be built here)"},
                "e2e": {"value": value, "unit": "s/q-point", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def normwise(a, b):
    w = 0.0
    for i in range(b.shape[2]):
        for j in range(b.shape[3]):
            d = np.abs(b[:, :, i, j]).max()
            if d:
                w = max(w, float(np.abs(a[:, :, i, j] - b[:, :, i, j]).max() / d))
    return w


def run_gpu(args):
    from respackdev_gb300 import build
    from respackdev_gb300 import chiqw as rp
    build.build()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811
        dist.init_process_group("gloo")
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    tmp = tempfile.mkdtemp(prefix="rp_bench_")
    try:
        t_prep = prepare(tmp, args.case)
        em = frequencies()
        params = rp.default_params(precision=rp.PREC_FP16X3, fft_box=FFT_BOX, device=dev, **RUN_PARAMS)
        t0 = time.time()
        ctx = rp.Context(tmp, params, em)
        t_setup = time.time() - t0
        info = ctx.info()
        npair_full = info.n_occ * info.n_vir
        K = npair_full * info.ntk
        # q points of this rank (weak scaling: every rank takes its own q points), Gamma excluded
        qs = step_q_list(ctx.L.rp_num_qirr(ctx._h), rank, world, args.warmup, args.steps)
        timed = qs[args.warmup:]
        for iq in qs[: args.warmup]:
            ctx.chi0_q(iq, fetch=False)
            ctx.epsinv_q(fetch=False)
        # --- device-resident timing ---
        launches0 = ctx.kernel_launches()
        if dist:
            dist.barrier()
        stage = np.zeros(5)
        tcg = 0.0
        alg_flops = 0.0
        ngs = []
        with ClockSampler(dev) as clk:
            t0 = time.perf_counter()
            for iq in timed:
                ctx.chi0_q(iq, fetch=False)
                st1 = ctx.stage_times()
                ctx.epsinv_q(fetch=False)
                st2 = ctx.stage_times()
                stage += np.array([st1[0], st1[1], st1[2], st2[3], st1[4]])
                tcg += ctx.tc_gram_seconds()
                ngs.append(ctx.ng)
            elapsed = time.perf_counter() - t0
        launches = ctx.kernel_launches() - launches0
        for ng_q in ngs:
            alg_flops += 8.0 * ng_q * ng_q * K * info.nen
        if dist:
            import torch
            t = torch.tensor([elapsed], dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            elapsed = float(t.item())
        value = elapsed / (args.steps * world)
        # --- end to end through the C ABI with host buffers, the same timed q points ---
        h2d0, d2h0 = ctx.transfer_bytes()
        t0 = time.perf_counter()
        for iq in timed:
            ctx.chi0_q(iq, fetch=True)
            ctx.epsinv_q(fetch=True)
        e2e = (time.perf_counter() - t0) / args.steps
        h2d1, d2h1 = ctx.transfer_bytes()
        h2d, d2h = (h2d1 - h2d0) // args.steps, (d2h1 - d2h0) // args.steps
        ctx.close()
        # --- plain FP64 path and the errors of the fast path on a pair sample of one q ---
        iq0 = timed[0]
        plain = err = eps_err = inv_err = None
        sample_pairs = 96
        if not args.no_plain:
            base = dict(fft_box=FFT_BOX, device=dev, max_pairs=sample_pairs, **RUN_PARAMS)
            with rp.Context(tmp, rp.default_params(precision=rp.PREC_FP64, **base), em) as c64:
                chi64 = c64.chi0_q(iq0)
                s64 = c64.stage_times()
                eps64 = c64.epsinv_q()
                e64 = c64.stage_times()[3]
            with rp.Context(tmp, rp.default_params(precision=rp.PREC_FP16X3, **base), em) as cs:
                chis = cs.chi0_q(iq0)
                epss = cs.epsinv_q()
            with rp.Context(tmp, rp.default_params(precision=rp.PREC_FP16X3, eps_fp64=1, **base), em) as cf:
                cf.chi0_q(iq0, fetch=False)
                epsf = cf.epsinv_q()
            err = normwise(chis, chi64)
            eps_err = normwise(epss, eps64)
            inv_err = normwise(epss, epsf)
            plain = s64[4] * npair_full / sample_pairs + e64
        # --- roofline of the tensor-core contraction ---
        tflops_sus, tflops_burst, hbm, src = measured_peaks()
        achieved = alg_flops / tcg / 1e12 if tcg > 0 else None
        roof = {"bound": "tensor", "kernel": "tc_gram_kernel", "achieved": achieved, "peak": tflops_sus,
                "unit": "TFLOP/s", "frac": (achieved / tflops_sus) if achieved else None,
                "peak_source": f"{src} bf16 sustained", "traffic": profile_traffic(),
                "tensor_products_per_real_product": 6,
                "achieved_tensor_tflops": achieved * 6 if achieved else None,
                "algorithmic_flops_per_q": alg_flops / max(1, len(ngs)),
                "algorithmic_flops": "8 NG^2 K nen per q, each q's own NG, K = pairs x k"}
        # --- CPU baseline (rank 0, host cores, bounded sample) ---
        cpu = None
        if rank == 0 and not args.no_cpu and args.case == "full":
            nthr = os.cpu_count() or 1
            v, rep = cpu_baseline(tmp, nthr, nthr, em, iq0, max_k=max(1, info.ntk // 4))
            cpu = {"value": v, "unit": "s/q-point", "cores": nthr, "kind": "port",
                   "sample": f"q {iq0}, {rep.npair_last} of {rep.npair_full_last} band pairs over {rep.nk_used_last} "
                             f"of {rep.ntk} k points on {nthr} threads, scaled linearly"}
        clocks = clk.summary()
        ragged = None
        if rank == 0 and args.case == "full" and not args.no_ragged:
            ragged = run_ragged(args, steps=min(args.steps, 3), warmup=1, emit=False)
        if rank == 0:
            line = {"metric": METRIC,
                    "value": value, "unit": "s/q-point", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                    "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": False, "scaling": "weak",
                    "vs_baseline": None, "dtype": "fp16x3-split tensor contraction, f32 pair densities, f32-series weights "
                             "(f64 closed forms near resonance), f32 Gauss-Jordan + float-pair Newton eps^-1",
                    "data": "synthetic (seeded generator, dir-wfn files)",
                    "config": workload_config(info.ntk, info.ncb, npair_full, ngs[0], info.nen, info.fft_box, timed,
                                              world) | ({} if args.case == "full" else {"workload": WORKLOAD + "_small"}),
                    "ng_per_step": ngs, "npw_max": info.ntg,
                    "plain_fp64_s_per_q": plain, "speedup_vs_plain_fp64": (plain / value) if plain else None,
                    "plain_fp64_sample": f"{sample_pairs} of {npair_full} pairs on q {iq0}, scaled linearly",
                    "plain_fp64_note": "the plain FP64 kernel forms the full complex chi (8 real flops per G, G', "
                                       "K, w); the split path forms the upper halves of two real symmetric Gram "
                                       "matrices of size 2 NG per w (also 8 NG^2 real flops per K and w), so both "
                                       "do the algorithmic count",
                    "chi_rel_err_vs_fp64": err,
                    "epsinv_rel_err_vs_fp64": eps_err,
                    "epsinv_mixed_vs_fp64_inverse_same_chi": inv_err,
                    "stage_seconds_per_q": {"tetra": stage[0] / args.steps, "pair_density": stage[1] / args.steps,
                                            "contraction": stage[2] / args.steps, "eps_inverse": stage[3] / args.steps},
                    "setup_seconds": t_setup, "input_generation_seconds": t_prep,
                    "roofline": roof, "clocks": clocks,
                    "e2e": {"value": e2e, "unit": "s/q-point", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                            "note": "all timed q points again through the C ABI with host result buffers; "
                                    "wave functions uploaded once per run (setup_seconds)"},
                    "gpu_launches": launches, "cpu_baseline": cpu, "ragged": ragged}
            print(json.dumps(line), flush=True)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
        if dist:
            dist.destroy_process_group()


# --- ragged batch: many cells' chi0 problems in one tensor-core launch ---------

RAGGED_CELLS = 12


def ragged_specs(seed=7, ncell=RAGGED_CELLS):
    """Seeded cells of the ragged workload: fcc/bcc/sc with a in [8, 14] bohr,
    k meshes 3^3..6^3, 60-300 bands (8 occupied), wave-function cutoff 12-24 Ry
    (raised where the sphere would hold fewer than 1.3x the bands, or to 1.5x
    the dielectric cutoff), a target dielectric sphere of 40-400 G reached by
    the dielectric cutoff, and 4-16 frequencies (half real 0-30 eV, half
    imaginary)."""
    from respackdev_gb300 import synth
    rng = np.random.default_rng(seed)
    vol_of = {"fcc": 0.25, "bcc": 0.5, "sc": 1.0}
    cells = []
    for i in range(ncell):
        lat = ("fcc", "bcc", "sc")[i % 3]
        a = float(rng.uniform(8.0, 14.0))
        nk = int(rng.integers(3, 7))
        nb = int(rng.integers(60, 301))
        ecut = float(rng.uniform(12.0, 24.0))
        vol = vol_of[lat] * a ** 3
        npw = lambda e: vol * e ** 1.5 / (6 * np.pi ** 2)
        while npw(ecut) < 1.3 * nb:
            ecut *= 1.1
        ng = int(rng.integers(40, 401))
        ecut_eps = (6 * np.pi ** 2 * ng / vol) ** (2.0 / 3.0)
        ecut = max(ecut, 1.5 * ecut_eps)  # the dielectric sphere stays well inside the density's
        nen = int(rng.integers(4, 17))
        nre = (nen + 1) // 2
        em = np.concatenate([np.linspace(0.0, 30.0, nre),
                             1j * np.linspace(30.0 / max(1, nen - nre), 30.0, nen - nre)]) / AU
        spec = synth.SynthSpec(lattice=lat, a=a, nk=(nk, nk, nk), nbands=nb, nocc=8, ecut_psi=ecut,
                               seed=1000 + i, wan_lo=9, wan_hi=11, shuffle_g=False)
        cells.append((spec, ecut_eps, em))
    return cells


def _make_cell(args):
    root, spec = args
    from respackdev_gb300 import synth
    synth.make_case(root, spec)
    return root


def run_ragged(args, steps=None, warmup=None, emit=True):
    """One step = chi0 of every problem of the ragged workload (two q points of
    each of the 12 cells) through rp_chi0_batch: preparation per problem, one
    grouped tensor-core launch and the assembly in one CUDA graph.  The same
    problems through rp_chi0_q one by one are timed beside it.  Prints the
    line (emit) and returns it."""
    steps = args.steps if steps is None else steps
    warmup = args.warmup if warmup is None else warmup
    import concurrent.futures as cf
    import multiprocessing as mp
    tmp = tempfile.mkdtemp(prefix="rp_ragged_")
    try:
        cells = ragged_specs()
        roots = [os.path.join(tmp, f"cell{i:02d}") for i in range(len(cells))]
        for r in roots:
            os.makedirs(r)
        t0 = time.time()
        # generate the cells in spawned processes (safe after GPU calls, unlike
        # forked ones), one BLAS thread each (the workers inherit the environment)
        blas = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")
        saved = {k: os.environ.get(k) for k in blas}
        os.environ.update({k: "1" for k in blas})
        try:
            with cf.ProcessPoolExecutor(max_workers=min(8, os.cpu_count() or 1),
                                        mp_context=mp.get_context("spawn")) as ex:
                list(ex.map(_make_cell, [(r, c[0]) for r, c in zip(roots, cells)]))
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
        gen = time.time() - t0
        from respackdev_gb300 import chiqw as rp
        rp.load()
        ctxs = []
        for r, (spec, ecut_eps, em) in zip(roots, cells):
            p = rp.default_params(precision=rp.PREC_FP16X3, ecut_for_eps=ecut_eps, green_func_delt=0.2721, flg_crpa=1)
            ctxs.append(rp.Context(r, p, em))
        probs, shapes = [], []
        for i, (c, (spec, _, em)) in enumerate(zip(ctxs, cells)):
            nq = c.L.rp_num_qirr(c._h)
            qs = [1, nq // 2 + 1] if i % 3 == 0 else [2, nq // 2 + 1]
            for iq in qs:
                ng, nd = c.q_dims(iq)
                inf = c.info()
                probs.append((c, iq))
                shapes.append({"cell": i, "lattice": spec.lattice, "a": round(spec.a, 3), "nk": spec.nk[0],
                               "bands": spec.nbands, "npw_max": inf.ntg, "q": iq, "ng": ng, "ndir": nd,
                               "nen": inf.nen, "npair": inf.n_occ * inf.n_vir})
        for _ in range(max(1, warmup)):
            rp.chi0_batch(probs, graph=True, fetch=False)
        launches0 = sum(c.kernel_launches() for c in ctxs)
        t0 = time.perf_counter()
        secs = np.zeros(3)
        for _ in range(steps):
            _, s = rp.chi0_batch(probs, graph=True, fetch=False)
            secs += s
        batch = (time.perf_counter() - t0) / steps
        launches = (sum(c.kernel_launches() for c in ctxs) - launches0) // steps
        t0 = time.perf_counter()
        seq_gram = 0.0
        for _ in range(steps):
            for c, iq in probs:
                c.chi0_q(iq, fetch=False)
                seq_gram += c.tc_gram_seconds()
        seq = (time.perf_counter() - t0) / steps
        seq_gram /= steps
        n = len(probs)
        line = {"metric": "chiqw ragged batch s/problem (all w), 12 cells in one grouped launch",
                "value": batch / n, "unit": "s/problem", "n_gpus": 1, "steps": steps, "warmup": warmup,
                "higher_is_better": False, "dtype": "fp16x3-split tensor contraction, f32 pair densities",
                "data": "synthetic (seeded generator, 12 cells)",
                "config": {"workload": "chiqw_ragged_12cells", "problems": n, "cells": len(cells)},
                "sequential_s_per_problem": seq / n, "speedup_vs_sequential": seq / batch,
                "sequential_gram_device_seconds": seq_gram,
                "batch_seconds": {"prepare": secs[0] / steps, "graph_device": secs[1] / steps,
                                  "finish": secs[2] / steps},
                "gram_launches_per_batch": 1, "gpu_launches_per_batch": int(launches),
                "tuned_shapes": rp.tuned_shapes(), "input_generation_seconds": gen, "shapes": shapes}
        if emit:
            print(json.dumps(line), flush=True)
        for c in ctxs:
            c.close()
        return line
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def run_large(args):
    """The large end-to-end workload on one GPU: fcc a = 15.84 bohr, 10x10x10 k
    (47 irreducible points of the cubic group in dat.sample-k), 1000 bands
    (8 occupied: 7936 band pairs), 31.7 Ry (about 2980 plane waves), 48^3 box,
    dielectric cutoff 25.8 Ry (about 2180 G), 30 frequencies (15 real 0-30 eV,
    15 imaginary on a Gauss-Legendre grid), FP16x3.  The real-space functions
    of all 1000 bands would take 885 GB, so the occupied bands stay resident and
    each pair batch transforms its virtual bands into a window.  A step is one q
    point; the q points timed are a stated subset of the 47.  The first timed
    q point's dir-eps is written (its dat.epsqw.600 record is above 2 GiB, in
    gfortran's subrecords) and read back."""
    from respackdev_gb300 import build
    from respackdev_gb300 import chiqw as rp
    from respackdev_gb300 import synth
    build.build()
    tmp = tempfile.mkdtemp(prefix="rp_large_")
    try:
        t0 = time.time()
        synth.make_case(tmp, synth.CASES["large"])
        gen = time.time() - t0
        x, _ = np.polynomial.legendre.leggauss(15)
        em = np.concatenate([np.linspace(0.0, 30.0, 15), 1j * 15.0 * (x + 1.0)]) / AU
        params = rp.default_params(precision=rp.PREC_FP16X3, fft_box=(48, 48, 48), ecut_for_eps=25.8,
                                   green_func_delt=0.2721, flg_crpa=1)
        t0 = time.time()
        ctx = rp.Context(tmp, params, em)
        setup = time.time() - t0
        info = ctx.info()
        qs = list(range(2, 2 + max(1, args.steps)))
        per_q, stages, ngs = [], [], []
        tflops_sus, _, _, src = measured_peaks()
        alg = 0.0
        tcg = 0.0
        with ClockSampler(0) as clk:
            for iq in qs:
                t0 = time.perf_counter()
                ctx.chi0_q(iq, fetch=False)
                st1 = ctx.stage_times()
                ctx.epsinv_q(fetch=False)
                per_q.append(time.perf_counter() - t0)
                st2 = ctx.stage_times()
                stages.append({"tetra": st1[0], "pair_density": st1[1], "contraction": st1[2], "eps_inverse": st2[3]})
                ngs.append(ctx.ng)
                tcg += ctx.tc_gram_seconds()
                alg += 8.0 * ctx.ng * ctx.ng * info.n_occ * info.n_vir * info.ntk * info.nen
        t0 = time.perf_counter()
        ctx.write_q()
        write_s = time.perf_counter() - t0
        rec = os.path.join(tmp, "dir-eps", "q%03d" % qs[-1], "dat.epsqw.600")
        nbytes = ngs[-1] * ngs[-1] * info.nen * 16
        ok_size = os.path.getsize(rec) == nbytes + 8 * ((nbytes + 2147483638) // 2147483639)
        with open(rec, "rb") as f:
            first_marker = int(np.frombuffer(f.read(4), dtype="<i4")[0])
        achieved = alg / tcg / 1e12 if tcg > 0 else None
        line = {"metric": "chiqw s/q-point (all w), large end-to-end workload", "value": float(np.mean(per_q)),
                "unit": "s/q-point", "n_gpus": 1, "steps": len(qs), "warmup": 0, "higher_is_better": False,
                "dtype": "fp16x3-split tensor contraction, f32 pair densities, f32-series/f64 weights",
                "data": "synthetic (seeded generator, 47 irreducible k of the cubic group)",
                "config": {"workload": "chiqw_10x10x10k_1000b", "ntk": info.ntk, "nk_irr": info.nk_irr,
                           "nbands": info.ncb, "npair": info.n_occ * info.n_vir, "npw_max": info.ntg,
                           "ng": ngs, "nen": info.nen, "fft_box": list(info.fft_box), "q_points": qs},
                "seconds_per_q": per_q, "stage_seconds": stages, "setup_seconds": setup,
                "input_generation_seconds": gen, "device_bytes": info.device_bytes,
                "roofline": {"bound": "tensor", "kernel": "tc_gram_kernel", "achieved": achieved, "peak": tflops_sus,
                             "unit": "TFLOP/s", "frac": achieved / tflops_sus if achieved else None,
                             "peak_source": f"{src} bf16 sustained"},
                "eps_record": {"q": qs[-1], "bytes": nbytes, "file_size_ok": ok_size,
                               "first_marker_negative": first_marker < 0, "write_seconds": write_s},
                "clocks": clk.summary()}
        print(json.dumps(line), flush=True)
        ctx.close()
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison")
    ap.add_argument("--no-ragged", action="store_true", help="skip the ragged-batch leg of the default line")
    ap.add_argument("--case", default="full", choices=["full", "small", "ragged", "large"],
                    help="small: 4x4x4 k, 100 bands, same kernels (for profiler captures); "
                         "ragged: 12 cells' chi0 problems in one grouped launch; "
                         "large: 10x10x10 k, 1000 bands, 48^3 box, about 2180 G (a q subset)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.case == "ragged":
        run_ragged(args)
    elif args.case == "large":
        run_large(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
