"""Benchmark of the Kohn-Sham XC build on one GB300 (one JSON line on stdout).

Workload: cyclo[18]carbon, restricted B3LYP / def2-TZVP (558 functions),
SG-2 grid (140 220 points, 2048 blocks).  A step is one XC build: density
(rho, grad rho) -> B3LYP functional -> E_xc -> V_xc, on an SCF-shaped
density matrix resident in HBM.  Synthetic geometry and density (seeded).

  python bench.py [--steps K] [--warmup W] [--precision mixed|fp64]
  python bench.py --impl reference   # the CPU XC path (oracle port of the
                                     # reference's per-block einsum loops)

Under torchrun (N > 1) every rank runs an independent replica of the same
build (the path does not need a collective: replicas only).
"""
import argparse
import json
import tempfile
import os
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "XC grid-pts/s (one B3LYP/def2-TZVP XC build of C18 on SG-2)"
UNIT = "grid-points/s"


def workload(name="c18"):
    from chinium_gb300 import molecules as M
    if name == "fe4s4":
        Z, xyz = M.fe4s4()
        return dict(name="Fe4S4 UKS TPSS/def2-TZVP SG-3, multiplicity 9", Z=Z, xyz=xyz, basis="def2-tzvp",
                    grid="SG-3", functional="TPSS", ids=[202, 231], nspin=2, nocc=(88, 80),
                    metric="XC grid-pts/s (one UKS TPSS/def2-TZVP XC build of Fe4S4 on SG-3)")
    Z, xyz = M.c18()
    return dict(name="C18 RKS B3LYP/def2-TZVP SG-2", Z=Z, xyz=xyz, basis="def2-tzvp", grid="SG-2",
                functional="B3LYP", ids=[402], nspin=1, nocc=54, metric=METRIC)


def model_density(nbasis, nocc, seed=0):
    """Closed-shell SCF-shaped total density 2 C C^T from random orthonormal
    orbitals mixed onto a diagonal occupation profile (keeps rho > 0)."""
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(nbasis, nocc)) * 0.05
    A[np.arange(nocc), np.arange(nocc)] += 1.0
    Q, _ = np.linalg.qr(A)
    return 2.0 * Q @ Q.T


def workload_density(wl, nbasis):
    """The workload's density matrices (row-major n x n, one per spin):
    restricted 2 C C^T, or per-spin C_s C_s^T of an open-shell occupation."""
    if wl["nspin"] == 1:
        return [model_density(nbasis, wl["nocc"])]
    return [0.5 * model_density(nbasis, no, seed=k) for k, no in enumerate(wl["nocc"])]


def max_over_ranks(t, world, device):
    """The slowest rank's time, the whole job's clock when every rank runs an
    independent replica (all-reduce MAX of one FP64 scalar on the process
    group; NCCL on the GPUs, gloo in the CPU tests); world 1 returns t."""
    if world <= 1:
        return t
    import torch
    import torch.distributed as dist
    x = torch.tensor([t], dtype=torch.float64, device=device)
    dist.all_reduce(x, op=dist.ReduceOp.MAX)
    return float(x.item())


def whole_job_rate(world, units_per_rank_step, steps, t_max):
    """Units all ranks processed per second: weak scaling, every rank handles
    units_per_rank_step per step, over the slowest rank's time."""
    return world * units_per_rank_step * steps / t_max


def clocks_start(path):
    try:
        f = open(path, "w")
        p = subprocess.Popen(
            ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
             "--format=csv,noheader,nounits", "-lms", "200"], stdout=f, stderr=subprocess.DEVNULL)
        return p, f
    except Exception:
        return None, None


def clocks_stop(p, f, path):
    if p is None:
        return None
    p.terminate()
    try:
        p.wait(timeout=5)
    except Exception:
        p.kill()
    f.close()
    rows = []
    for ln in open(path):
        t = [x.strip() for x in ln.split(",")]
        if len(t) >= 9:
            try:
                rows.append((float(t[1]), float(t[2]), t[5:9]))
            except ValueError:
                pass
    if not rows:
        return None
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
    return {"sm_mhz": float(np.median([r[0] for r in rows])), "sm_max_mhz": max(r[1] for r in rows),
            "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def fp64_gemm_peak(torch):
    """cuBLAS DGEMM throughput (TFLOP/s), the FP64 denominator of the plain path."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    return 2 * n ** 3 / best / 1e12


class CpuArm:
    """The oracle (CPU restatement of the reference's per-block einsum loops,
    OpenMP over blocks) on the first sample_blocks blocks of the same
    workload (0 = every block): grid, blocks and AO values set up once.
    Throughput counts the real (unpadded) points of the blocks built."""

    def __init__(self, wl, D, sample_blocks, threads):
        from oracle import oracle as O
        basis = O.Basis(wl["Z"], wl["xyz"], wl["basis"])
        px, py, pz, w = O.grid_points(wl["Z"], wl["xyz"], wl["grid"])
        allb = O.padded_blocks(px, py, pz, w)
        ranges = O.block_ranges(len(px))
        self.total = len(allb)
        nblk = sample_blocks if 0 < sample_blocks < len(allb) else len(allb)
        blocks = allb[:nblk]
        g = O.OracleGrid.__new__(O.OracleGrid)
        g.basis = basis
        g.blocks = blocks
        g.ao = [basis.ao(b[0], b[1], b[2], 1) for b in blocks]
        g.npoints = sum(len(b[0]) for b in blocks)
        self.g, self.D, self.ids, self.threads = g, D, wl["ids"], threads
        self.nspin = wl["nspin"]
        self.npad = g.npoints
        self.nreal = int(sum(n for _, n in ranges[:nblk]))
        self.whole = nblk == len(allb)
        self.E, self.F = g.build(D, wl["ids"], self.nspin, nblocks=1, nthreads=threads)  # warm

    def step(self):
        """One timed build of the sample: (real grid-points/s, seconds); keeps E_xc, V_xc."""
        t = time.perf_counter()
        self.E, self.F = self.g.build(self.D, self.ids, self.nspin, nthreads=self.threads)
        dt = time.perf_counter() - t
        return self.nreal / dt, dt

    def describe(self, dt):
        return {"unit": UNIT, "cores": self.threads, "kind": "port",
                "sample": "%d of %d blocks (%d real points), one build, %.2f s" % (
                    len(self.g.blocks), self.total, self.nreal, dt)}


def cpu_baseline(wl, D, sample_blocks, threads):
    arm = CpuArm(wl, D, sample_blocks, threads)
    v, dt = arm.step()
    return dict(value=v, **arm.describe(dt)), arm


def run_reference(args):
    """The reference arm: the oracle port of the reference's CPU XC build
    (per-block einsum loops, OpenMP over blocks on every host thread) on the
    same workload, one whole build per step.  Nothing of the product is
    loaded: the basis size comes from the oracle's own basis."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    wl = workload(args.workload if args.workload in ("c18", "fe4s4") else "c18")
    nb = O.Basis(wl["Z"], wl["xyz"], wl["basis"]).nbasis
    Dm = workload_density(wl, nb)
    threads = os.cpu_count() or 1
    arm = CpuArm(wl, Dm, args.ref_blocks, threads)
    vals, times = [], []
    for i in range(args.warmup + args.steps):
        v, dt = arm.step()
        if i >= args.warmup:
            vals.append(v)
            times.append(dt)
    t = float(np.sum(times))
    v = arm.nreal * len(times) / t
    cb = dict(value=v, **arm.describe(float(np.median(times))))
    line = {"impl": "reference", "metric": wl["metric"], "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / len(times) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": wl["name"], "npoints": arm.nreal,
                                            "blocks": "%d of %d" % (len(arm.g.blocks), arm.total),
                                            "whole_build": arm.whole, "E_xc": arm.E},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def mixed_roofline(info, kms, stage, peaks, family, nspin):
    """Roofline of the dominant mixed kernel against both of its limits.
    Tensor: algorithmic FLOPs ÷ CUDA-event duration, from the grid's unit
    counts: density 2*128*128*64 per unit — a full pass (rho + grad rho, GGA /
    meta-GGA) has units_full units, a symmetric pass (rho of LDA, each of the
    three tau components) units_sym; V_xc 2*128^3 per (item, tile) job and
    component (components 1-3 only on jobs with I <= J).  The tensor core
    executes 6x that (three-term split cross products).  HBM: algorithmic
    bytes ÷ duration — per kept (function, point) pair the A operand (6 B of
    BF16 planes, or 4 B FP32 when split in-kernel) plus the FP32 values the
    density epilogue contracts (4 B per component), or the V kernel's L and R
    operands per component; plus the FP64 outputs (densities per point, one
    128 x 128 W partial per V item).  The reported bound is the roof with the
    larger algorithmic fraction; both sub-objects are in the line."""
    unit = 2.0 * 128 * 128 * 64
    if family == 0:
        fl_den = info["mixed_units_sym"] * unit * nspin
    elif family == 1:
        fl_den = info["mixed_units_full"] * unit * nspin
    else:
        fl_den = (info["mixed_units_full"] + 3 * info["mixed_units_sym"]) * unit * nspin
    jobs = info["mixed_fock_jobs"] + (3 * info["mixed_fock_tau_jobs"] if family >= 2 else 0)
    fl_fock = jobs * 2.0 * 128 ** 3 * nspin  # one fock_tc launch per spin; kms[4] sums them
    ms_den, ms_fock = kms[0], kms[4]
    # kernels on pre-split BF16 planes (density16 / fock16) or converting FP32 tiles in-kernel
    presplit = bool(info.get("mixed_presplit"))
    kd, kf = ("density16", "fock16") if presplit else ("density_tc", "fock_tc")
    # algorithmic HBM bytes per build: every operand byte read once, outputs written once
    rp = info["mixed_rows"] * 128  # kept (function, point) pairs of all tiles
    G = info["mixed_tiles"] * 128
    a_op = 6 if presplit else 4    # A operand bytes per element (BF16 planes or FP32)
    if family == 0:
        by_den = rp * (a_op + 4) + G * 16
    elif family == 1:
        by_den = rp * (a_op + 16) + G * 64
    else:
        by_den = rp * (a_op + 16) + G * 64 + 3 * (rp * (a_op + 4) + G * 32)
    ncv = 4 if family >= 2 else 1
    by_fock = rp * ncv * (a_op + (6 if presplit else 4)) + info.get("mixed_fock_items", 0) * 16384 * 8
    by_den, by_fock = by_den * nspin, by_fock * nspin
    dom, dom_ms, fl, by = (kd, ms_den, fl_den, by_den) if ms_den >= ms_fock else (kf, ms_fock, fl_fock, by_fock)
    achieved = fl / (dom_ms / 1e3) / 1e12
    peak = peaks.get("bf16_tflops", 1900.0)
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    hbm = by / (dom_ms / 1e3) / 1e9
    tensor = {"achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
              "executed_tflops": 6 * achieved, "executed_frac": 6 * achieved / peak,
              "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst) -- of measured"}
    memory = {"achieved": hbm, "peak": hbm_peak, "unit": "GB/s", "frac": hbm / hbm_peak,
              "algorithmic_bytes_per_build": by, "peak_source": "MEASURED_PEAKS.json hbm_gbs -- of measured"}
    # the binding roof: the one whose algorithmic fraction is larger (the kernel is closest to it);
    # the tensor pipe's executed fraction (6 split products) is reported beside it
    hbm_bound = memory["frac"] >= tensor["frac"]
    main = memory if hbm_bound else tensor
    return {"bound": "hbm" if hbm_bound else "tensor", "kernel": dom, "achieved": main["achieved"],
            "peak": main["peak"], "unit": main["unit"], "frac": main["frac"], "traffic": None,
            "peak_source": main["peak_source"], "tensor": tensor, "hbm": memory,
            "executed_tensor_tflops": 6 * achieved, "executed_frac": 6 * achieved / peak,
            "kernel_ms": {kd + " (+split_d, combine)": kms[0], "functional": kms[1], "energy": kms[2],
                          ("prep16" if kd == "density16" else "prep_z"): kms[3], kf: kms[4], "wsum": kms[5]},
            "stage_ms": {"density": stage[0], "functional": stage[1], "energy": stage[2], "fock": stage[3]}}


def time_builds(torch, grid, xc, dD, dE, dV, precision, steps, stream):
    """Device time of `steps` back-to-back builds on the build stream (s)."""
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(steps):
        grid.build_device(xc, dD, dE, dV, precision)
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / 1e3


ALK_METRIC = "XC grid-pts/s (batched r2SCAN/def2-SVP XC build of 64 alkanes on SG-2)"


def run_alkanes(args):
    """64 linear alkanes C_nH_(2n+2), n ~ U{1..20} (seed 0), restricted
    r2SCAN/def2-SVP on SG-2: every molecule's tiles in one persistent launch
    per stage, replayed from a CUDA graph; the autotuner picks the screening
    threshold, the V work-item length and the tile formation first.  FP64
    per-molecule builds on the same densities give the accuracy and the plain
    path's time."""
    import ctypes
    import torch
    import chinium_gb300 as cg
    from chinium_gb300 import molecules as M
    from chinium_gb300._lib import check, lib
    torch.cuda.set_device(0)
    mols = M.alkane_batch(64, seed=0)
    bases = [cg.Basis(Z, xyz, "def2-svp") for Z, xyz in mols]
    xc = cg.ExchangeCorrelation().Read("R2SCAN")
    PMX, P64 = cg.PRECISION_MIXED, cg.PRECISION_FP64
    t0 = time.perf_counter()
    bg = cg.BatchGrid(bases, "SG-2")
    bg.setType(xc.type)
    t_grid = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    bg.set_stream(stream.cuda_stream)
    Ds = [[model_density(b.nbasis, sum(Z) // 2, seed=m)] for m, ((Z, _), b) in enumerate(zip(mols, bases))]
    Dpk = bg._pack(Ds)
    nm = len(mols)
    tune = None
    if not args.no_tune:
        t0 = time.perf_counter()
        tune = bg.tune(xc, Ds, e_tol=1e-7, v_tol=1e-5, reps=2)
        tune["seconds"] = time.perf_counter() - t0
    dD = torch.from_numpy(Dpk).cuda()
    dE = torch.zeros(nm, dtype=torch.float64, device="cuda")
    dV = torch.zeros(bg.packed_size, dtype=torch.float64, device="cuda")
    t0 = time.perf_counter()
    bg.build_device(xc, dD, dE, dV, PMX)
    stream.synchronize()
    t_first = time.perf_counter() - t0
    for _ in range(args.warmup):
        bg.build_device(xc, dD, dE, dV, PMX)
    stream.synchronize()
    Emx = dE.cpu().numpy().copy()
    Vmx = dV.cpu().numpy().copy()
    info = bg.info()
    bg.profile(True)
    bg.build_device(xc, dD, dE, dV, PMX)
    stage = bg.stage_ms()
    kms = bg.kernel_ms()
    bg.profile(False)
    clk_dir = os.environ.get("XC_BENCH_OUT") or tempfile.gettempdir()
    os.makedirs(clk_dir, exist_ok=True)
    clk_path = os.path.join(clk_dir, "clocks_alkanes.csv")
    cp, cf = clocks_start(clk_path)
    time.sleep(0.4)
    t_dev = time_builds(torch, bg, xc, dD, dE, dV, PMX, args.steps, stream)
    clocks = clocks_stop(cp, cf, clk_path)
    # end to end through the public host-buffer call
    Dh = torch.from_numpy(Dpk).pin_memory()
    Vh = torch.zeros(bg.packed_size, dtype=torch.float64).pin_memory()
    Eh = torch.zeros(nm, dtype=torch.float64).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        check(lib().xc_build(bg._h, xc._h, ctypes.c_void_p(Dh.data_ptr()), 1, PMX, ctypes.c_void_p(Eh.data_ptr()),
                             ctypes.c_void_p(Vh.data_ptr())))
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    # plain FP64 path, molecule by molecule, same densities
    nfp = nm if args.fp64_mols <= 0 else min(nm, args.fp64_mols)
    t64, dEs, dVs = 0.0, [], []
    for m in range(nfp):
        g = cg.Grid(bases[m], "SG-2")
        g.setType(xc.type)
        g.getAO(0)
        g.set_stream(stream.cuda_stream)
        n = bases[m].nbasis
        d1 = torch.from_numpy(np.ascontiguousarray(Ds[m][0].T)).cuda()
        e1 = torch.zeros(1, dtype=torch.float64, device="cuda")
        v1 = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        g.build_device(xc, d1, e1, v1, P64)
        t64 += time_builds(torch, g, xc, d1, e1, v1, P64, 1, stream)
        o = int(bg.offsets[m])
        dEs.append(abs(float(e1.item()) - Emx[m]))
        dVs.append(float(np.abs(v1.cpu().numpy().ravel() - Vmx[o:o + n * n]).max()))
        del g
    G = int(bg.npoints.sum())
    Gfp = int(bg.npoints[:nfp].sum())
    value = G * args.steps / t_dev
    plain = Gfp / t64
    peaks = measured_peaks()
    roof = mixed_roofline(info, kms, stage, peaks, 2, 1)
    line = {"metric": ALK_METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3 (split) + f64 accumulation", "data": "synthetic",
            "config": {"workload": "64 alkanes C_nH_(2n+2), n ~ U{1..20} seed 0, RKS r2SCAN/def2-SVP SG-2, batched",
                       "molecules": nm, "npoints": G, "mixed_tiles": info["mixed_tiles"],
                       "nbasis_total": int(sum(b.nbasis for b in bases)),
                       "l2": "inputs larger than L2 (FP32 AO store + Z %.1f GB)" % (info["mixed_store_bytes"] / 1e9),
                       "batched_builds_per_s": args.steps / t_dev,
                       "molecule_builds_per_s": nm * args.steps / t_dev,
                       "grid_setup_s": t_grid, "first_build_s": t_first, "tuner": tune,
                       "plain_fp64_molecules": nfp, "plain_fp64_pts_per_s": plain,
                       "speedup_vs_plain_fp64": value / plain,
                       "max_abs_dE_xc_vs_fp64": max(dEs), "max_abs_dV_xc_vs_fp64": max(dVs)},
            "e2e": {"value": G * args.steps / t_e2e, "unit": UNIT, "h2d_bytes_per_step": 8 * bg.packed_size,
                    "d2h_bytes_per_step": 8 * (bg.packed_size + nm)},
            "gpu_launches": args.steps * info["mixed_launches"], "roofline": roof, "clocks": clocks}
    print(json.dumps(line), flush=True)


SCF_METRIC = "SCF wall time to 1e-8 Eh, (H2O)_8 RKS PBE/def2-SVP SG-2, mixed + learned guess"


def scf_water_legs(nmols, molecules=None, grid="SG-2", legs_cfg=None):
    """Full Kohn-Sham SCFs to 1e-8 Eh (PBE/def2-SVP) of seeded held-out water
    octamers (disjoint from the guess's training seeds) or of the given
    molecules: (a) plain FP64 XC builds from the SAP guess -- with the
    reference's unscreened blocks and with block screening 1e-11 -- and from
    the learned guess, and (b) incremental mixed builds from the learned guess
    (its SAP base on the tensor cores; references from float-float densities
    with a tensor-core V), plus the other combinations.  Integrals, the overlap
    metric and the grids are shared setup (repulsion integrals computed on the
    GPU and resident in HBM); the timed SCF includes the guess and every
    iteration (XC build, J/K contraction, DIIS, orbital update).  Returns the
    per-leg means and the speed-ups."""
    import chinium_gb300 as cg
    from chinium_gb300 import guess as G
    from chinium_gb300 import molecules as M
    from chinium_gb300.scf import run_scf
    mols = molecules or M.water_clusters(nmols, seed=424242, kmin=8, kmax=8)
    model = G.load(G.DEFAULT_WEIGHTS)
    # (XC precision, guess, reference build of the incremental mixed SCF, FP64 block screening).
    # Screening 0 is the reference's semantics (every function in every block); 1e-11 drops the shells
    # below 1e-11 on a block, which leaves E_xc unchanged to 1e-14 Eh here and makes FP64 builds 2.4x faster.
    legs_cfg = legs_cfg or {
        "fp64_sap": ("fp64", "sap", "fp64", 0.0), "fp64_sap_screened": ("fp64", "sap", "fp64", 1e-11),
        "fp64_learned": ("fp64", "learned", "fp64", 0.0), "fp64_learned_screened": ("fp64", "learned", "fp64", 1e-11),
        "mixed_sap": ("mixed", "sap", "density", 1e-11), "mixed_learned": ("mixed", "learned", "density", 1e-11),
        "mixed_learned_unscreened_anchor": ("mixed", "learned", "density", 0.0)}
    legs = {k: [] for k in legs_cfg}
    dE = []
    t_setup = 0.0
    xc = cg.ExchangeCorrelation().Read("PBE")
    for Z, xyz in mols:
        kw = dict(functional="PBE", grid=grid, jk_device="engine")
        t0 = time.perf_counter()
        ctxs = {}
        for scr in sorted({v[3] for v in legs_cfg.values()}):  # integrals shared; one grid per screening
            ctx = {k: v for k, v in next(iter(ctxs.values())).items() if not k.startswith("grid")} if ctxs else None
            warm = run_scf(Z, xyz, precision="fp64", guess="core", max_iter=1, context=ctx, screen=scr, **kw)
            ctxs[scr] = warm.context
            ctxs[scr]["grid"].build(xc, [warm.D[0]], precision=cg.PRECISION_MIXED)  # mixed tiles, AO planes
        t_setup += time.perf_counter() - t0
        res = {}
        for leg, (prec, gs, anchor, scr) in legs_cfg.items():
            ctx = ctxs[scr]
            t0 = time.perf_counter()
            guess = "sap" if gs == "sap" else G.guess_density(model, Z, xyz, ctx, precision=prec)
            r = run_scf(Z, xyz, precision=prec, guess=guess, context=ctx, anchor=anchor, screen=scr, **kw)
            wall = time.perf_counter() - t0
            assert r.converged
            legs[leg].append({"wall": wall, "iters": r.iterations, "E": r.energy, "xc_s": r.timings["xc"],
                              "jk_s": r.timings["jk"], "diag_s": r.timings["diag"]})
            res[leg] = r.energy
        dE.append(abs(res["mixed_learned"] - res["fp64_sap"]))
        for leg in legs:
            legs[leg][-1]["dE"] = abs(res[leg] - res["fp64_sap"])
    summ = {k: {"wall_s": float(np.mean([x["wall"] for x in v])), "iterations": float(np.mean([x["iters"] for x in v])),
                "xc_s": float(np.mean([x["xc_s"] for x in v])), "jk_s": float(np.mean([x["jk_s"] for x in v])),
                "diag_s": float(np.mean([x["diag_s"] for x in v])),
                "max_abs_dE_vs_fp64_sap": float(max(x["dE"] for x in v))} for k, v in legs.items()}
    value = summ["mixed_learned"]["wall_s"]
    best = min((v["wall_s"], k) for k, v in summ.items() if k.startswith("fp64"))
    return {"molecules": len(mols), "legs": summ, "setup_s_per_molecule": t_setup / len(mols),
            "mixed_learned_s": value, "speedup_vs_plain_fp64_sap": summ["fp64_sap"]["wall_s"] / value,
            "speedup_vs_screened_fp64_sap": summ["fp64_sap_screened"]["wall_s"] / value
            if "fp64_sap_screened" in summ else None,
            "best_fp64_leg": best[1], "speedup_vs_best_fp64": best[0] / value,
            "max_abs_dE_total_vs_plain_fp64": float(max(dE))}


def run_scf_water(args):
    """The SCF line of held-out water octamers (scf_water_legs)."""
    import torch
    torch.cuda.set_device(0)
    r = scf_water_legs(args.scf_mols)
    value = r["mixed_learned_s"]
    line = {"metric": SCF_METRIC, "value": value, "unit": "s", "n_gpus": 1, "steps": r["molecules"], "warmup": 0,
            "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x3 (split) + f64 accumulation (XC); f64 elsewhere", "data": "synthetic",
            "config": dict({"workload": "(H2O)_8 water clusters (seed 424242), RKS PBE/def2-SVP SG-2, SCF to 1e-8 Eh"},
                           **r)}
    print(json.dumps(line), flush=True)


def scf_summaries():
    """SCF results carried by the default line (a few seconds each): the
    (H2O)_8 SG-2 legs on two held-out octamers, the single water of the
    plain-path configuration (PBE/def2-SVP SG-1 from the SAP guess, FP64)
    beside its mixed + learned SCF, and the learned guess on 24 held-out
    clusters of 2-8 waters (SG-1, mixed SCFs, SAP vs learned start)."""
    import types
    from chinium_gb300 import molecules as M
    from chinium_gb300 import learn_guess as LG
    from chinium_gb300 import guess as G
    out = {"scf_water8_sg2": scf_water_legs(2)}
    h2o = scf_water_legs(1, molecules=[M.h2o()], grid="SG-1", legs_cfg={
        "fp64_sap": ("fp64", "sap", "fp64", 0.0), "fp64_learned": ("fp64", "learned", "fp64", 0.0),
        "mixed_learned": ("mixed", "learned", "density", 0.0)})
    out["scf_h2o_sg1"] = h2o
    a = types.SimpleNamespace(test=24, kmin=2, kmax=8, test_kmax=8, functional="PBE", jk="engine", precision="mixed")
    t0 = time.perf_counter()
    rows = LG.evaluate(G.load(G.DEFAULT_WEIGHTS), a, lambda s: None)
    out["learned_guess_24_heldout_sg1"] = dict(LG.summarize(rows), eval_s=time.perf_counter() - t0)
    return out


JK_METRIC = "Coulomb (J) builds/s, (H2O)8 def2-SVP, repulsion integrals on the GPU (in-core)"


def run_jk(args):
    """The SCF caller's Coulomb / exchange engine on one held-out (H2O)_8
    (seed 424242, def2-SVP, n = 192): integrals computed once on the GPU and
    kept in HBM (set-up), then a step is one J build of the dense Coulomb
    operator (pack, GEMV, unpack) on a density resident in HBM; K builds are
    timed beside it.  The operator is held as float-float pairs (8 bytes per
    element, 48-bit significands) and the GEMV runs on the FP32 pipe, so its
    roof is HBM: the operator's bytes over the build's CUDA-event time
    against the measured HBM rate."""
    import ctypes
    import torch
    import chinium_gb300 as cg
    from chinium_gb300 import molecules as M
    from chinium_gb300._lib import check, lib
    from chinium_gb300.scf import JKEngine
    if int(os.environ.get("RANK", "0")) != 0:
        return
    torch.cuda.set_device(0)
    Z, xyz = M.water_clusters(1, seed=424242, kmin=8, kmax=8)[0]
    b = cg.Basis(Z, xyz, "def2-svp")
    n = b.nbasis
    t0 = time.perf_counter()
    jk = JKEngine(b, threshold=1e-12)
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    info = jk.info()
    D = torch.from_numpy(model_density(n, sum(Z) // 2)[None].copy()).cuda()
    J = torch.empty((1, n, n), dtype=torch.float64, device="cuda")
    K = torch.empty((1, n, n), dtype=torch.float64, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    st = jk.stream

    def timed(steps, with_k):
        for _ in range(max(args.warmup, 1)):
            check(lib().xc_jk_build_device(jk._h, 1, p(D), p(J), p(K) if with_k else None))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(steps):
            check(lib().xc_jk_build_device(jk._h, 1, p(D), p(J), p(K) if with_k else None))
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / steps

    t_j = timed(args.steps, False)
    t_jk = timed(max(args.steps // 4, 1), True)
    npair = n * (n + 1) // 2
    npair += npair & 1
    op_bytes = 8.0 * npair * npair
    peaks = measured_peaks()
    hbm = op_bytes / t_j / 1e9
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    line = {"metric": JK_METRIC, "value": 1.0 / t_j, "unit": "builds/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_j * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32x2 (float-float operator and density, FP64 sums)", "data": "synthetic",
            "config": {"workload": "(H2O)_8 (seed 424242) RKS def2-SVP, J of one density per step", "nbasis": n,
                       "integrals": info, "setup_s": t_setup, "j_plus_k_ms": t_jk * 1e3,
                       "l2": "inputs larger than L2 (dense Coulomb operator %.2f GB)" % (op_bytes / 1e9)},
            "roofline": {"bound": "hbm", "kernel": "coulomb_gemv_kernel", "achieved": hbm, "peak": hbm_peak,
                         "unit": "GB/s", "frac": hbm / hbm_peak, "traffic": None,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs -- of measured"}}
    print(json.dumps(line), flush=True)


def run_c18_mixed(args):
    """C18 B3LYP/def2-TZVP SG-2: grid, AO store and tiles set up, then only
    mixed-precision builds (the kernels of the headline, for profiling)."""
    import torch
    import chinium_gb300 as cg
    if int(os.environ.get("RANK", "0")) != 0:
        return
    torch.cuda.set_device(0)
    wl = workload("c18")
    b = cg.Basis(wl["Z"], wl["xyz"], wl["basis"])
    xc = cg.ExchangeCorrelation().Read(wl["functional"])
    g = cg.Grid(b, wl["grid"])
    g.setType(xc.type)
    g.getAO(0)
    if args.v_operands:  # 1: operands split inside the kernels (as for batches whose planes do not fit)
        g.set_mixed_config(v_operands=args.v_operands)
    D = model_density(b.nbasis, wl["nocc"])
    for _ in range(args.warmup):
        g.build(xc, [D], precision=cg.PRECISION_MIXED)
    g.profile(True)
    g.build(xc, [D], precision=cg.PRECISION_MIXED)
    kms = g.kernel_ms()
    g.profile(False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        E, _ = g.build(xc, [D], precision=cg.PRECISION_MIXED)
    t = (time.perf_counter() - t0) / args.steps
    print(json.dumps({"metric": wl["metric"] + ", host-buffer mixed builds only", "value": g.info()["npoints"] / t,
                      "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                      "dtype": "bf16x3 (split) + f64 accumulation", "data": "synthetic",
                      "config": {"workload": wl["name"], "E_xc": E, "v_operands": args.v_operands,
                                 "kernel_ms": dict(zip(("density", "functional", "energy", "v_operand",
                                                        "v_partials", "v_reduction"), kms))}}), flush=True)


C18_SCF_METRIC = "SCF wall time to 1e-8 Eh, C18 RKS B3LYP/def2-TZVP SG-2, mixed vs plain FP64 XC"


def run_c18_scf(args):
    """cyclo[18]carbon, restricted B3LYP/def2-TZVP (558 functions) on SG-2:
    full Kohn-Sham SCFs to 1e-8 Eh from the SAP guess, Coulomb and exact
    exchange from the library's GPU integrals (4.9e9 unique integrals of 8.1e7
    shell quartets, computed in FP64 once in the shared set-up and kept in
    HBM as float-float pairs).  Legs: the plain FP64 XC build
    every iteration (per-block shell screening 1e-11, the same energies as
    unscreened to 1e-14 Eh) and incremental tensor-core XC builds (references
    from FP64 densities).  The timed SCF includes the guess and every
    iteration (XC build, J/K contraction, DIIS, orbital update)."""
    import torch
    from chinium_gb300 import molecules as M
    from chinium_gb300.scf import run_scf
    if int(os.environ.get("RANK", "0")) != 0:
        return
    torch.cuda.set_device(0)
    Z, xyz = M.c18()
    kw = dict(basis="def2-tzvp", functional="B3LYP", grid="SG-2", jk_device="engine", screen=1e-11)
    t0 = time.perf_counter()
    warm = run_scf(Z, xyz, precision="fp64", guess="core", max_iter=1, **kw)
    ctx = warm.context
    t_setup = time.perf_counter() - t0
    jk_info = ctx["jk"].info()
    legs = {}
    for leg, prec in (("fp64", "fp64"), ("mixed", "mixed")):
        t0 = time.perf_counter()
        r = run_scf(Z, xyz, precision=prec, guess="sap", context=ctx, anchor="density", **kw)
        wall = time.perf_counter() - t0
        legs[leg] = {"wall_s": wall, "iterations": r.iterations, "converged": bool(r.converged), "E": r.energy,
                     "xc_s": r.timings["xc"], "jk_s": r.timings["jk"], "orbital_update_s": r.timings["diag"]}
    dE = abs(legs["mixed"]["E"] - legs["fp64"]["E"])
    value = legs["mixed"]["wall_s"]
    line = {"metric": C18_SCF_METRIC, "value": value, "unit": "s", "n_gpus": 1, "steps": 1, "warmup": 0,
            "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x3 (split) + f64 accumulation (XC); f64 integrals, J/K in float-float (48-bit) "
                     "on the FP32 pipe, f64 DIIS", "data": "synthetic",
            "config": {"workload": "C18 RKS B3LYP/def2-TZVP SG-2, SCF to 1e-8 Eh from the SAP guess",
                       "setup_s": t_setup, "integrals": jk_info, "legs": legs,
                       "speedup_vs_plain_fp64": legs["fp64"]["wall_s"] / value,
                       "abs_dE_total_mixed_vs_fp64": dE}}
    print(json.dumps(line), flush=True)


def run_gradient(args):
    """C18 RKS B3LYP/def2-TZVP SG-2: the XC nuclear gradient with the grid fixed
    (getDensitySkeleton + getEnergyGrad, FP64) through the C ABI, host buffers;
    one step is one gradient (upload of D, FP64 density and functional, the
    gradient kernel, reduction by atom).  Unscreened blocks (the reference's
    BasisList) and shells screened at 1e-11 (the same gradient to 1e-12).
    Roofline of the gradient kernel: FP64 FLOPs of its two products per block
    (T = phi D and U = Z D: 2 * 2 g n_b^2), the Z operand (8 g n_b) and the
    contraction with the AO gradients and Hessians (27 g n_b), over the
    kernel's CUDA-event time, against the cuBLAS DGEMM rate measured here."""
    import torch
    import chinium_gb300 as cg

    if int(os.environ.get("RANK", "0")) != 0:
        return
    wl = workload("c18")
    basis = cg.Basis(wl["Z"], wl["xyz"], wl["basis"])
    n = basis.nbasis
    xc = cg.ExchangeCorrelation().Read(wl["functional"])
    D = model_density(n, wl["nocc"])
    out = {}
    for key, thr in (("unscreened", 0.0), ("screened_1e-11", 1e-11)):
        g = cg.Grid(basis, wl["grid"], screen_threshold=thr)
        g.setType(xc.type)
        g.getAO(1)
        for _ in range(max(args.warmup, 1)):
            G = g.getEnergyGrad(xc, [D])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            G = g.getEnergyGrad(xc, [D])
        t = (time.perf_counter() - t0) / args.steps
        g.profile(True)
        g.getEnergyGrad(xc, [D])
        ms = g.stage_ms()
        g.profile(False)
        pts = g.points()
        nb = np.asarray(pts["nb"], dtype=np.float64)
        ng = np.asarray(pts["ng"], dtype=np.float64)
        flops = float(np.sum(4 * ng * nb * nb + 35 * ng * nb))
        out[key] = {"ms_per_gradient": t * 1e3, "kernel_ms": ms[2], "density_ms": ms[0], "functional_ms": ms[1],
                    "kernel_fp64_tflops": flops / (ms[2] * 1e-3) / 1e12, "grad": G}
        if thr > 0:
            # the Hessian's skeleton V_xc terms on the same grid (getFockSkeleton + getFockU<s_t>, 3 N_atoms
            # matrices each): one warm-up call, one timed
            g.getFockSkeleton(xc, [D])
            t0 = time.perf_counter()
            FS, FU = g.getFockSkeleton(xc, [D])
            out[key]["fock_skeleton_ms"] = (time.perf_counter() - t0) * 1e3
            out[key]["fock_skeleton_matrices"] = int(FS.shape[1])
            del FS, FU
        del g
    peak = fp64_gemm_peak(torch)
    sc = out["screened_1e-11"]
    diff = float(np.abs(out["unscreened"]["grad"] - sc["grad"]).max())
    for v in out.values():
        v.pop("grad")
    line = {"metric": "XC nuclear gradients/s (C18 B3LYP/def2-TZVP SG-2, grid fixed, FP64)",
            "value": 1e3 / sc["ms_per_gradient"], "unit": "gradients/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sc["ms_per_gradient"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "C18 RKS B3LYP/def2-TZVP SG-2, XC gradient (getDensitySkeleton + getEnergyGrad)",
                       "legs": out, "max_abs_dgrad_screened_vs_unscreened": diff,
                       "l2": "inputs larger than L2 (AO store with Hessians, 10 components)"},
            "e2e": {"value": 1e3 / sc["ms_per_gradient"], "unit": "gradients/s", "h2d_bytes_per_step": 8 * n * n,
                    "d2h_bytes_per_step": 0},
            "roofline": {"bound": "fp64", "kernel": "grad_fp64_kernel", "achieved": sc["kernel_fp64_tflops"],
                         "peak": peak, "unit": "TFLOP/s", "frac": sc["kernel_fp64_tflops"] / peak,
                         "traffic": None, "peak_source": "cuBLAS DGEMM 4096^3 measured in this run"}}
    print(json.dumps(line), flush=True)


def response_cpu_baseline(wl, D, U, sample_blocks=256, threads=None):
    """The oracle's response (the reference's getDensityU + getFockU<u_t>
    restated, with its FP64 ground state and second derivatives per block),
    OpenMP over blocks on every host thread as the reference bins its blocks,
    on the first sample_blocks blocks of the same grid for one perturbation,
    scaled to one matrix over the whole grid."""
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    basis = O.Basis(wl["Z"], wl["xyz"], wl["basis"])
    px, py, pz, w = O.grid_points(wl["Z"], wl["xyz"], wl["grid"])
    allb = O.padded_blocks(px, py, pz, w)
    g = O.OracleGrid.__new__(O.OracleGrid)
    g.basis = basis
    g.blocks = allb[:sample_blocks]
    g.ao = [basis.ao(b[0], b[1], b[2], 1) for b in g.blocks]
    t = time.perf_counter()
    g.build_response(D[None], U[None, None], wl["ids"], 1, nthreads=threads)
    dt = time.perf_counter() - t
    per_matrix = dt * len(allb) / len(g.blocks)
    return {"value": 1.0 / per_matrix, "unit": "matrices/s", "cores": threads, "kind": "port",
            "sample": "%d of %d blocks, one perturbation, %.2f s (one matrix over the grid: %.1f s)" % (
                len(g.blocks), len(allb), dt, per_matrix)}


def run_response(args):
    """C18 RKS B3LYP/def2-TZVP SG-2 (shells screened at 1e-11), the response
    work of one CPSCF iteration for the 3 N_atoms = 54 symmetric perturbations
    of a Hessian: the ground state (getDensity, Evaluate("ev"), Evaluate("f"))
    is prepared once, as the reference does before its CPSCF loop
    (Restricted/Hess.cpp:79); a step is getDensityU + getFockU<u_t> of the 54
    matrices through the C ABI with host buffers (uploads of D_U, response
    densities and V_U, downloads inside the timed region), as each iteration of
    CoupledPerturbed.cpp:131-134.  The FP64 path runs once on the same input
    for the speed-up and the accuracy; the fused call (ground state included)
    is timed beside it."""
    import ctypes
    import torch
    import chinium_gb300 as cg
    from chinium_gb300._lib import check, lib

    if int(os.environ.get("RANK", "0")) != 0:
        return
    wl = workload("c18")
    basis = cg.Basis(wl["Z"], wl["xyz"], wl["basis"])
    n = basis.nbasis
    g = cg.Grid(basis, wl["grid"], screen_threshold=1e-11)
    xc = cg.ExchangeCorrelation().Read(wl["functional"])
    g.setType(xc.type)
    g.getAO(0)
    P64, PMX = cg.PRECISION_FP64, cg.PRECISION_MIXED
    prec = P64 if args.precision == "fp64" else PMX
    nmat = 3 * len(wl["Z"])
    D = model_density(n, wl["nocc"])
    rng = np.random.default_rng(11)
    A = rng.normal(size=(nmat, n, n)) * 0.01
    Dst = g._stack([D])
    Du = np.ascontiguousarray((A + A.transpose(0, 2, 1))[None])  # symmetric: column-major = row-major
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    g.getDensity([D])
    xc.Evaluate("ev", g)
    xc.Evaluate("f", g)

    def step(p, F):
        check(lib().xc_grid_set_response_precision(g._h, p))
        check(lib().xc_grid_get_density_u(g._h, ptr(Du), 1, nmat))
        check(lib().xc_grid_get_fock_u(g._h, ptr(F)))

    F = np.zeros_like(Du)
    for _ in range(max(args.warmup, 1)):
        step(prec, F)
    clk = os.path.join(os.environ.get("XC_BENCH_OUT") or tempfile.gettempdir(), "clocks_resp.csv")
    cp, cf = clocks_start(clk)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step(prec, F)
    t = (time.perf_counter() - t0) / args.steps
    clocks = clocks_stop(cp, cf, clk)
    roof = None
    if prec == PMX:
        # CUDA events around the first matrix's kernels of one more iteration: its density16
        # launch is the dominant kernel; the tiles, and so the algorithmic bytes, are the build's
        g.profile(True)
        step(prec, F)
        ms = g.stage_ms()
        g.profile(False)
        info = g.info()
        kms = [ms[0], 0.0, 0.0, ms[1], ms[2], ms[3]]
        roof = mixed_roofline(info, kms, [ms[0], 0.0, 0.0, ms[1] + ms[2] + ms[3]], measured_peaks(), xc.type, 1)
        roof["kernel_ms"] = {"split_d + density16 + combine": ms[0], "response_coef + prep16": ms[1],
                             "fock16": ms[2], "wsum": ms[3]}
        roof.pop("stage_ms", None)
        tf = os.path.join(REPO, "profiles", "traffic_c18_b3lyp_sg2.json")
        if os.path.exists(tf) and roof["kernel"] == "density16":
            tr = json.load(open(tf)).get("dram_bytes_per_launch", {}).get("density16")
            roof["traffic"] = tr
            roof["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of density16 on the same "
                                      "tiles (C18 build), profiles/traffic_c18_b3lyp_sg2.json")
    cfg = {"workload": "C18 RKS B3LYP/def2-TZVP SG-2, 54 symmetric perturbations, one CPSCF iteration",
           "precision": args.precision, "nbasis": n, "nmat": nmat, "grid": "shells screened at 1e-11",
           "ground_state": "fp64 (density, functional, second derivatives), prepared once before the steps",
           "l2": "inputs larger than L2 (D_U of a step 134 MB; AO stores)"}
    Ff = np.zeros_like(Du)
    t1 = time.perf_counter()
    check(lib().xc_build_response(g._h, xc._h, ptr(Dst), 1, prec, nmat, ptr(Du), ptr(Ff)))
    cfg["fused_call_ms_incl_ground_state"] = (time.perf_counter() - t1) * 1e3
    if not args.no_fp64 and prec == PMX:
        F64 = np.zeros_like(Du)
        g.getDensity([D])
        xc.Evaluate("ev", g)
        xc.Evaluate("f", g)
        t1 = time.perf_counter()
        step(P64, F64)
        t64 = time.perf_counter() - t1
        cfg.update({"fp64_ms_per_step": t64 * 1e3, "speedup_vs_fp64": t64 / t,
                    "max_abs_dV_U_vs_fp64": float(np.abs(F - F64).max()), "max_abs_V_U": float(np.abs(F64).max())})
    line = {"metric": "XC response V_U matrices/s (C18 B3LYP/def2-TZVP SG-2, 54 perturbations per CPSCF iteration)",
            "value": nmat / t, "unit": "matrices/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x3 (split) + f64 accumulation" if prec == PMX else "f64", "data": "synthetic",
            "config": cfg,
            "e2e": {"value": nmat / t, "unit": "matrices/s", "h2d_bytes_per_step": int(Du.nbytes),
                    "d2h_bytes_per_step": int(F.nbytes)},
            "gpu_launches": nmat * 7 if prec == PMX else 4,  # per matrix: split_d, density16, combine, response_coef, prep16, fock16, wsum
            "roofline": roof, "clocks": clocks}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = response_cpu_baseline(wl, D, Du[0, 0])
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--cpu-blocks", type=int, default=0,
                    help="blocks of the workload in the CPU baseline of this arm (0 = all: one whole build)")
    ap.add_argument("--ref-blocks", type=int, default=0,
                    help="blocks per step of the --impl reference arm (0 = all: one whole build per step)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="c18", choices=["c18", "fe4s4", "alkanes64", "scf-water", "c18-response",
                                                         "c18-gradient", "c18-scf", "jk-water8", "c18-mixed"])
    ap.add_argument("--no-fp64", action="store_true", help="c18-response: skip the FP64 comparison")
    ap.add_argument("--scf-mols", type=int, default=4)
    ap.add_argument("--fp64-mols", type=int, default=0, help="alkanes64: molecules checked in FP64 (0 = all)")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--no-scf", action="store_true", help="c18: leave out the SCF and learned-guess results")
    ap.add_argument("--v-operands", type=int, default=0, choices=[0, 1, 2],
                    help="c18-mixed: operand form of the tensor-core kernels (0 by free memory, 1 split in-kernel, 2 pre-split)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "alkanes64":
        return run_alkanes(args)
    if args.workload == "scf-water":
        return run_scf_water(args)
    if args.workload == "c18-response":
        return run_response(args)
    if args.workload == "c18-gradient":
        return run_gradient(args)
    if args.workload == "c18-scf":
        return run_c18_scf(args)
    if args.workload == "jk-water8":
        return run_jk(args)
    if args.workload == "c18-mixed":
        return run_c18_mixed(args)

    import ctypes
    import torch
    import chinium_gb300 as cg
    from chinium_gb300._lib import check, lib

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    wl = workload(args.workload)
    ns = wl["nspin"]
    basis = cg.Basis(wl["Z"], wl["xyz"], wl["basis"])
    n = basis.nbasis
    grid = cg.Grid(basis, wl["grid"], nspin=ns, screen_threshold=0.0)
    xc = cg.ExchangeCorrelation(spin=ns).Read(wl["functional"])
    grid.setType(xc.type)
    grid.getAO(0)
    stream = torch.cuda.Stream()
    grid.set_stream(stream.cuda_stream)
    P64, PMX = cg.PRECISION_FP64, cg.PRECISION_MIXED
    precision = P64 if args.precision == "fp64" else PMX

    Dl = workload_density(wl, n)
    Dst = np.ascontiguousarray(np.stack([d.T for d in Dl]))
    D = Dl[0] if ns == 1 else Dl[0] + Dl[1]
    Dsp = Dl
    dD = torch.from_numpy(Dst).cuda()
    dE = torch.zeros(1, dtype=torch.float64, device="cuda")
    dV = torch.zeros((ns, n, n), dtype=torch.float64, device="cuda")

    # plain FP64 path on the same density: reference numbers and throughput
    grid.build_device(xc, dD, dE, dV, P64)
    stream.synchronize()
    E64, V64 = float(dE.item()), dV.clone()
    plain_steps = max(1, args.plain_steps)
    t_plain = time_builds(torch, grid, xc, dD, dE, dV, P64, plain_steps, stream)
    # the FP64 path with per-block shell screening at 1e-11 (the reference keeps
    # every function in every block): reported beside the unscreened numbers
    gs = cg.Grid(basis, wl["grid"], nspin=ns, screen_threshold=1e-11)
    gs.setType(xc.type)
    gs.getAO(0)
    gs.set_stream(stream.cuda_stream)
    gs.build_device(xc, dD, dE, dV, P64)
    stream.synchronize()
    E64s = float(dE.item())
    t_plain_s = time_builds(torch, gs, xc, dD, dE, dV, P64, plain_steps, stream)
    del gs
    # the FP64 XC nuclear gradient (grid fixed; LDA / GGA only), on a grid with AO Hessians
    t_grad = None
    if xc.type <= 1:
        gg = cg.Grid(basis, wl["grid"], nspin=ns, screen_threshold=0.0)
        gg.setType(xc.type)
        gg.getAO(1)
        Dl = [D] if ns == 1 else Dsp
        gg.getEnergyGrad(xc, Dl)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            gg.getEnergyGrad(xc, Dl)
        t_grad = (time.perf_counter() - t0) / 3 * 1e3
        del gg
    # the FP64 response V_U (Evaluate("f") + getDensityU + getFockU<u_t>) for the
    # 3 N_atoms perturbations a CPSCF / Hessian step carries, on the screened grid
    resp = None
    if xc.type <= 1:
        gr = cg.Grid(basis, wl["grid"], nspin=ns, screen_threshold=1e-11)
        gr.setType(xc.type)
        gr.getAO(0)
        nmat = 3 * len(wl["Z"])
        rng = np.random.default_rng(11)
        Dl = [D] if ns == 1 else Dsp
        U = []
        for _ in range(ns):
            A = rng.normal(size=(nmat, n, n)) * 0.01
            U.append(list(A + A.transpose(0, 2, 1)))
        resp = {"nmat": nmat, "grid": "shells screened at 1e-11", "host_buffers": "C-ABI call, column-major host arrays",
                "ground_state": "fp64 (density, functional, second derivatives)"}
        # column-major host buffers prepared once: the timed region is the C-ABI call
        # (upload of D and D_U, FP64 ground state, response, download of V_U)
        from chinium_gb300._lib import lib as _xl, check as _xchk
        import ctypes
        Dst_r = gr._stack(Dl)
        Du, _ = gr._stack_u(U)
        Du2, _ = gr._stack_u([u[:2] for u in U])
        _ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        out = {}
        for prec, key in ((P64, "fp64"), (PMX, "mixed")):
            F2 = np.zeros_like(Du2)
            _xchk(_xl().xc_build_response(gr._h, xc._h, _ptr(Dst_r), ns, prec, 2, _ptr(Du2), _ptr(F2)))  # warm-up
            F = np.zeros_like(Du)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _xchk(_xl().xc_build_response(gr._h, xc._h, _ptr(Dst_r), ns, prec, nmat, _ptr(Du), _ptr(F)))
            t_resp = (time.perf_counter() - t0) * 1e3
            out[key] = F
            resp[key] = {"ms": t_resp, "ms_per_matrix": t_resp / nmat}
        resp["speedup_mixed_vs_fp64"] = resp["fp64"]["ms"] / resp["mixed"]["ms"]
        resp["max_abs_dV_U_mixed_vs_fp64"] = float(np.abs(out["mixed"] - out["fp64"]).max())
        resp["max_abs_V_U"] = float(np.abs(out["fp64"]).max())
        del gr, U, out

    for _ in range(args.warmup):
        grid.build_device(xc, dD, dE, dV, precision)
    stream.synchronize()
    Emx, Vmx = float(dE.item()), dV.clone()
    info = grid.info()

    # stage timing of one build (CUDA events on the build stream)
    grid.profile(True)
    grid.build_device(xc, dD, dE, dV, precision)
    stage = grid.stage_ms()
    kms = grid.kernel_ms() if precision == PMX else None
    grid.profile(False)

    clk_dir = os.environ.get("XC_BENCH_OUT") or tempfile.gettempdir()
    os.makedirs(clk_dir, exist_ok=True)
    clk_path = os.path.join(clk_dir, "clocks_bench.csv")
    cp, cf = clocks_start(clk_path) if rank == 0 else (None, None)
    time.sleep(0.4)
    if world > 1:
        torch.distributed.barrier()
    t_dev = time_builds(torch, grid, xc, dD, dE, dV, precision, args.steps, stream)
    if world > 1:
        torch.distributed.barrier()
    t_dev = max_over_ranks(t_dev, world, "cuda")
    clocks = clocks_stop(cp, cf, clk_path) if rank == 0 else None

    # end to end through the public host-buffer call: pinned D in, E and V out
    Dh = torch.from_numpy(Dst).pin_memory()
    Vh = torch.zeros((ns, n, n), dtype=torch.float64).pin_memory()
    Eh = ctypes.c_double()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        check(lib().xc_build(grid._h, xc._h, ctypes.c_void_p(Dh.data_ptr()), ns, precision, ctypes.byref(Eh),
                             ctypes.c_void_p(Vh.data_ptr())))
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(time.perf_counter() - t0, world, "cuda")

    G = info["npoints"]  # real points (the reference's padded blocks carry zero-weight copies)
    value = whole_job_rate(world, G, args.steps, t_dev)
    e2e = whole_job_rate(world, G, args.steps, t_e2e)
    plain = G * plain_steps / t_plain
    peaks = measured_peaks()

    if precision == PMX:
        roof = mixed_roofline(info, kms, stage, peaks, xc.type, ns)
        tf = os.path.join(REPO, "profiles", "traffic_c18_b3lyp_sg2.json")
        if args.workload == "c18" and os.path.exists(tf):
            with open(tf) as f:
                t = json.load(f)
            roof["traffic"] = t["dram_bytes_per_launch"].get(roof["kernel"])
            roof["traffic_source"] = "ncu dram__bytes_read.sum + dram__bytes_write.sum, profiles/traffic_c18_b3lyp_sg2.json"
    else:
        flops = 2.0 * info["screened_pairs"] * (G / info["nblocks"])
        ms_den, ms_fock = stage[0], stage[3]
        dom, dom_ms = ("density_fp64", ms_den) if ms_den >= ms_fock else ("fock_fp64", ms_fock)
        peak = fp64_gemm_peak(torch)
        achieved = flops / (dom_ms / 1e3) / 1e12
        roof = {"bound": "fp64", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": None,
                "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (no FP64 entry in MEASURED_PEAKS.json)",
                "stage_ms": {"density": stage[0], "functional": stage[1], "energy": stage[2], "fock": stage[3]}}

    line = {"metric": wl["metric"], "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if precision == P64 else "bf16x3 (split) + f64 accumulation",
            "data": "synthetic",
            "config": {"workload": wl["name"], "precision": args.precision, "npoints": info["npoints"],
                       "npoints_padded": info["npoints_padded"], "nblocks": info["nblocks"], "nbasis": n,
                       "mixed_tiles": info["mixed_tiles"],
                       "l2": "inputs larger than L2 (FP64 AO store %.2f GB; FP32 AO store + Z %.2f GB)"
                             % (info["ao_elements"] * 4 * 8 / 1e9, info["mixed_store_bytes"] / 1e9),
                       "xc_builds_per_s": args.steps / t_dev,
                       "plain_fp64_pts_per_s": plain, "plain_fp64_ms_per_build": t_plain / plain_steps * 1e3,
                       "speedup_vs_plain_fp64": value / world / plain,
                       "plain_fp64_screened_ms_per_build": t_plain_s / plain_steps * 1e3,
                       "speedup_vs_screened_fp64": (t_plain_s / plain_steps) / (t_dev / args.steps),
                       "abs_dE_xc_screened_vs_unscreened_fp64": abs(E64s - E64),
                       "xc_gradient_fp64_ms": t_grad,
                       "xc_response": resp,
                       "E_xc_fp64": E64, "E_xc": Emx if precision == PMX else E64,
                       "abs_dE_xc_vs_fp64": abs(Emx - E64),
                       "max_abs_dV_xc_vs_fp64": float((Vmx - V64).abs().max().item())},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 8 * ns * n * n,
                    "d2h_bytes_per_step": 8 * ns * n * n + 8},
            "gpu_launches": args.steps * (info["mixed_launches"] if precision == PMX else 4),
            "roofline": roof, "clocks": clocks}
    if rank == 0 and not args.no_cpu_baseline:
        cb, arm = cpu_baseline(wl, Dl, args.cpu_blocks, os.cpu_count() or 1)
        line["cpu_baseline"] = cb
        if arm.whole:
            # parity of the plain FP64 path with the oracle on this workload (same grid, basis,
            # functional and density): the plain path's bar is 1e-10 in both
            V64h = V64.cpu().numpy()
            line["config"]["abs_dE_xc_fp64_vs_oracle"] = abs(E64 - arm.E)
            line["config"]["max_abs_dV_xc_fp64_vs_oracle"] = float(max(
                np.abs(V64h[s_].T - arm.F[s_]).max() for s_ in range(ns)))
    if rank == 0 and args.workload == "c18" and not args.no_scf:
        line["scf"] = scf_summaries()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
