#!/usr/bin/env python3
"""Benchmark of the GBLUP / ssGBLUP hot path on GB300.

Workload (default ``--config c3``): single-step GBLUP on a pedigree of 200,000
animals over 10 discrete generations (500 sires x 10,000 dams per generation,
random mating, 5 % unknown parents), the last 20,000 genotyped at m = 50,000
SNPs (genotypes gene-dropped through the pedigree from base frequencies
U(0.01, 0.5), 2 % missing calls), h2 = 0.35, one record per animal, fixed
effects mean + 500-level herd-year.  H^-1 = A^-1 + [0; (0.95 G + 0.05 A22)^-1 -
A22^-1] with tuneG.  Seeded synthetic data of those shapes (no public dataset
exists).

Setup (untimed, phases reported): BED -> GRM on the tensor cores, Henderson
A^-1, A22 by the pedigree recursion, tuneG, blend and both FP64 inverses on
the device, mixed-model equations on the device.

Step: one AI-REML iteration -- the EM update with Hutchinson traces (one data
solve plus the reference's adaptive probe schedule, >= 32 Rademacher probes,
solved as multi-RHS blocks) -- followed by the REML gradient (the reference's
AI-REML score) at the iteration's starting point from 64 probes, whose first
probes are the iteration's own solves; every solve to relative residual 1e-10.
``value`` uses the mixed-precision solver (FP32 PCG bulk, FP64 refinement on
the true residual) with all inputs resident in HBM.  The plain FP64 path runs
the same number of steps from the same starting point; the variance
components, the final EBVs and the gradient of the two paths are compared.
``e2e`` runs the same iterations through the public C ABI from host buffers:
every iteration uploads the records, the design and A^-1 again and rebuilds
the MME, whose solves start from the previous MME's solutions.

``--impl reference`` times the CPU restatement of the path (FP64 PCG, numpy
with all host threads) and counts, in the run, the PCG iterations of the
reference's algorithm (one right-hand side at a time, each solve from zero).
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

METRIC = ("REML iter/s & PCG solves/s at relres 1e-10, mixed vs FP64, 1 GB300; "
          "GRM int8 TOPS")
UNIT = "REML iter/s"

_SS = dict(kind="ssgblup", n_gen=10, per_gen=20000, n_sires=500, n_dams=10000, p_unknown=0.05, n=20000,
           m=50000, p_lo=0.01, miss=0.02, var_a=0.35, var_e=0.65, levels=500, seed=3000)
CONFIGS = {
    # single-step GBLUP (the default line): REML iteration + gradient from 64 probes
    "c3": dict(_SS, name="ssgblup_ped200000_geno20000_m50000_hy500", grad_probes=64),
    # the same data, gradient from 256 probes
    "c4": dict(_SS, name="ssgblup_ped200000_geno20000_m50000_hy500_grad256", grad_probes=256),
    "c2": dict(name="gblup_n20000_m50000_cg200", n=20000, m=50000, p_lo=0.01, miss=0.02,
               var_a=0.3, var_e=0.7, levels=200, seed=2000, grad_probes=0),
    # profiling case: same generator, G^-1 block (268 MB FP32) still larger than L2
    "c2s": dict(name="gblup_n8192_m16384_cg200", n=8192, m=16384, p_lo=0.01, miss=0.02,
                var_a=0.3, var_e=0.7, levels=200, seed=2100, grad_probes=0),
    # plain GBLUP, the dense exact AI-REML step (dim < 5000, as the reference chooses)
    "c1": dict(name="gblup_n2000_m10000_sex2", n=2000, m=10000, p_lo=0.05, miss=0.01,
               var_a=0.4, var_e=0.6, levels=2, seed=1000, grad_probes=0, dense=True),
    # 96 independent GBLUPs, n ~ log-uniform [500, 8000], m ~ log-uniform
    # [5000, 40000], h2 ~ U(0.1, 0.6), mean + 10-level group; each one GRM +
    # eigen-bent G^-1 + REML (3 EM iterations), the batch sharing the GPU
    "c5": dict(name="batch96_gblup_n500-8000_m5000-40000", kind="batch", nprob=96, n_lo=500, n_hi=8000,
               m_lo=5000, m_hi=40000, levels=10, max_iter=3, workers=16, seed=5000, mt_n=10000, mt_m=20000),
}
# DRAM bytes (read + written) per launch of the block product from ncu captures at
# n = 8,192, scaled to a 20,000-row block by the block's bytes (x (20000 / 8192)^2):
# k_dense_tf32<64> (the GBLUP iteration's block, 33 columns) 282.9 MB -> 1.686e9, and
# k_dense_tf32<128, 80> (the iteration + gradient block, 65 columns) 278.4 MB -> 1.659e9
TRAFFIC_BYTES = {(20000, 64): 1.686e9, (20000, 128): 1.659e9}
# the reference's adaptive estimator with one thread checks after two batches of 16
REF_EM_PROBES = 32


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d["hbm_gbs"], d["bf16_tflops"], "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thr = threading.Thread(target=self._read, daemon=True)
            self.thr.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def build_data(cfg) -> dict:
    """Seeded synthetic inputs of a single-problem workload (host only): the
    BED, the records and fixed-effect design, and for ssGBLUP the pedigree and
    the genotyped rows (the last generation)."""
    from cosmicblup_gb300.design import fixed_design
    from cosmicblup_gb300.synth import (genetic_values, pedigree_breeding_values, simulate_bed,
                                        simulate_bed_gene_drop, simulate_gblup_records, simulate_pedigree)
    n, m, seed = cfg["n"], cfg["m"], cfg["seed"]
    d = {"sire": None, "dam": None, "gmap": None}
    if cfg.get("kind") == "ssgblup":
        sire, dam = simulate_pedigree(cfg["n_gen"], cfg["per_gen"], cfg["n_sires"], cfg["n_dams"],
                                      seed=seed + 1, p_unknown=cfg["p_unknown"])
        q = sire.size
        d["bed"], _ = simulate_bed_gene_drop(sire, dam, cfg["per_gen"], m, seed=seed, p_lo=cfg["p_lo"],
                                             miss=cfg["miss"])
        a = pedigree_breeding_values(sire, dam, cfg["var_a"], seed=seed + 2)
        rec = simulate_gblup_records(q, cfg["levels"], a, seed=seed + 3, var_e=cfg["var_e"])
        d.update(sire=sire, dam=dam, gmap=np.arange(q - n, q, dtype=np.int32))
    else:
        q = n
        d["bed"], _ = simulate_bed(n, m, seed=seed, p_lo=cfg["p_lo"], miss=cfg["miss"])
        g = genetic_values(d["bed"], n, m, seed=seed + 2, var_a=cfg["var_a"])
        rec = simulate_gblup_records(n, cfg["levels"], g, seed=seed + 3, var_e=cfg["var_e"])
    dsg = fixed_design(rec["cats"])
    d.update(rec=rec, p=dsg.p, rows=dsg.csr(), q=q)
    return d


def solves_per_step(cfg, em_probes: float) -> float:
    """Single right-hand-side solves of one step in the reference's algorithm:
    the EM iteration's data solve and probes, then for the gradient the score
    of run_aireml_step (its own data solve and the trace probes)."""
    s = 1.0 + em_probes
    if cfg.get("grad_probes"):
        s += 1.0 + cfg["grad_probes"]
    return s


def cpu_pcg_iteration_cost(WtW, Qd, p, lam, iters: int, seed: int = 0, Ainv=None, gmap=None) -> float:
    """Seconds per FP64 PCG iteration of the oracle on the operator W'W + lam [0; Qinv]
    with Qinv = Qd (dense), or Ainv + S Qd S^T (sparse Ainv, dense block Qd on
    the rows gmap) when Ainv is given.

    Runs a fixed number of iterations (tol = 0) with the block-Jacobi
    preconditioner; numpy/BLAS uses every host thread."""
    from oracle.mme import pcg
    dim = WtW.shape[0]
    matvec, prec = cpu_operator(WtW, Qd, p, lam, Ainv, gmap)
    rng = np.random.default_rng(seed)
    b = np.zeros(dim)
    b[p:] = rng.choice([-1.0, 1.0], size=dim - p)
    t0 = time.perf_counter()
    pcg(matvec, b, prec, tol=0.0, maxit=iters)
    dt = time.perf_counter() - t0
    return dt / (iters + 2)  # iterations + the initial and final residual matvecs


def cpu_operator(WtW, Qd, p, lam, Ainv=None, gmap=None):
    """(matvec, block-Jacobi preconditioner) of the FP64 MME operator on the host."""
    d = WtW.diagonal().copy()
    if Ainv is None:
        d[p:] += lam * np.diag(Qd)
    else:
        dq = Ainv.diagonal().copy()
        dq[gmap] += np.diag(Qd)
        d[p:] += lam * dq
    A11 = WtW[:p, :p].toarray()
    A11[np.diag_indices(p)] += max(1e-8 * np.abs(np.diag(A11)).max(), 1e-6)
    dinv = 1.0 / d[p:]

    def matvec(v):
        y = WtW @ v
        if Ainv is None:
            y[p:] += lam * (Qd @ v[p:])
        else:
            u = v[p:]
            qu = Ainv @ u
            qu[gmap] += Qd @ u[gmap]
            y[p:] += lam * qu
        return y

    def prec(v):
        r = np.empty_like(v)
        r[:p] = np.linalg.solve(A11, v[:p])
        r[p:] = dinv * v[p:]
        return r

    return matvec, prec


# ---------------------------------------------------------------------------
def run_reference(args, cfg):
    """The CPU restatement of the path on a bounded sample (rank 0 only).

    The reference itself cannot be built (its CMake needs Eigen 3 and zstd.h).
    Each step times PCG iterations of the oracle's FP64 block-Jacobi PCG (the
    reference's PCGSolver, one right-hand side, numpy/BLAS on every host thread)
    on the workload's full-size operator.  For ssGBLUP that operator has the
    pedigree's real Henderson A^-1 and the records' real W'W, while the dense
    block is a stand-in of its order, because the FP64 G and A22 inverses take
    longer than the run may.  The cost of an iteration does not depend on the
    block's values.  The PCG iterations per solve are counted in the run: the
    data right-hand side is solved from zero to relres 1e-10 on this operator,
    as the reference solves every probe.  One step of the workload is that many
    iterations times the solves of the reference's algorithm per step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if cfg.get("kind") == "batch":
        print(json.dumps({"impl": "reference", "unavailable":
                          f"the CPU port is timed on single-problem workloads only, not {cfg['name']}"}))
        return
    import scipy.sparse as sp
    from oracle.mme import MME, build_fixed_design, invert_psd_matrix, pcg, sparse_data_part
    t0 = time.perf_counter()
    d = build_data(cfg)
    rec, p, q, n = d["rec"], d["p"], d["q"], cfg["n"]
    _, orows, _ = build_fixed_design(rec["cats"])
    cores = os.cpu_count()
    setup = {"synthetic_data_s": time.perf_counter() - t0}
    lam = cfg["var_e"] / cfg["var_a"]
    if cfg.get("dense"):
        # the dense exact AI step of the oracle on the real problem (small: n = 2,000)
        from oracle.grm import vanraden_grm
        from oracle.reml import AIREML as OracleREML
        t0 = time.perf_counter()
        Gi = invert_psd_matrix(vanraden_grm(d["bed"], n, cfg["m"])["G"])
        om = MME(rec["y"], rec["aid"], orows, p, q)
        setup["grm_inverse_s"] = time.perf_counter() - t0
        o = OracleREML(om, Gi, 0.5, 0.5)
        for _ in range(args.warmup):
            o.dense_exact_step()
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            o.dense_exact_step()
            times.append(time.perf_counter() - t0)
        c = float(np.mean(times))
        value = 1.0 / c
        sample = f"oracle dense exact AI-REML step (numpy/BLAS on {cores} threads), {args.steps} steps timed"
        ms = c * 1e3
    else:
        rng = np.random.default_rng(7)
        WtW, W = sparse_data_part(rec["aid"], orows, p, q)
        Qd = rng.standard_normal((n, n)) * (1.0 / n)
        Qd = 0.5 * (Qd + Qd.T)
        Qd[np.diag_indices(n)] += 2.0
        Ainv = gmap = None
        if d["sire"] is not None:
            from oracle.ped import ainv_henderson
            t0 = time.perf_counter()
            ap, ac, av, _, _ = ainv_henderson(d["dam"], d["sire"])
            Ainv = sp.csr_matrix((av, ac, ap), shape=(q, q))
            gmap = d["gmap"]
            setup["ainv_s"] = time.perf_counter() - t0
        # PCG iterations per solve of the reference's algorithm, counted on this operator
        matvec, prec = cpu_operator(WtW, Qd, p, lam, Ainv, gmap)
        t0 = time.perf_counter()
        _, it_solve, rel, _ = pcg(matvec, W.T @ rec["y"], prec, tol=1e-10, maxit=20000)
        setup["count_solve_s"] = time.perf_counter() - t0
        per_step_iters = 10
        for _ in range(args.warmup):
            cpu_pcg_iteration_cost(WtW, Qd, p, lam, per_step_iters, Ainv=Ainv, gmap=gmap)
        costs = [cpu_pcg_iteration_cost(WtW, Qd, p, lam, per_step_iters, seed=s, Ainv=Ainv, gmap=gmap)
                 for s in range(args.steps)]
        c = float(np.mean(costs))
        solves = solves_per_step(cfg, REF_EM_PROBES)
        work = solves * (it_solve + 1)
        value = 1.0 / (c * work)
        ms = c * work * 1e3
        sample = (f"oracle FP64 PCG, {per_step_iters} iterations per step on the {q + p}-row operator "
                  f"(numpy/BLAS, {cores} threads; dense block a stand-in of order {n}); {it_solve} PCG "
                  f"iterations per solve counted in this run (data right-hand side from zero, relres "
                  f"{rel:.1e}); {solves:.0f} solves per step "
                  f"({1 + REF_EM_PROBES} EM" + (f" + {1 + cfg['grad_probes']} gradient" if cfg.get("grad_probes")
                                                  else "") + ")")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": cfg["name"], "precision": "fp64 (CPU restatement)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "setup": setup,
    }))


# ---------------------------------------------------------------------------
def run_batch(args, cfg):
    """Batched uneven GBLUPs (cbx_batch_reml): wall time of the whole batch,
    mixed precision and the plain FP64 path, many workers and one."""
    from cosmicblup_gb300 import BatchProblem, RemlConfig, batch_reml
    from cosmicblup_gb300.design import fixed_design
    from cosmicblup_gb300.mme import FP64, MIXED
    from cosmicblup_gb300.synth import genetic_values, simulate_bed, simulate_gblup_records
    from cosmicblup_gb300.vce import MODE_EM
    rng = np.random.default_rng(cfg["seed"])
    t0 = time.perf_counter()
    probs = []
    for i in range(cfg["nprob"]):
        n = int(round(np.exp(rng.uniform(np.log(cfg["n_lo"]), np.log(cfg["n_hi"])))))
        m = int(round(np.exp(rng.uniform(np.log(cfg["m_lo"]), np.log(cfg["m_hi"])))))
        h2 = rng.uniform(0.1, 0.6)
        bed, _ = simulate_bed(n, m, seed=cfg["seed"] + 10 * i, p_lo=0.01, miss=0.02)
        g = genetic_values(bed, n, m, seed=cfg["seed"] + 10 * i + 1, var_a=h2)
        rec = simulate_gblup_records(n, cfg["levels"], g, seed=cfg["seed"] + 10 * i + 2, var_e=1.0 - h2)
        d = fixed_design(rec["cats"])
        probs.append(BatchProblem(bed=bed, n=n, m=m, y=rec["y"], aid=rec["aid"], rows=d.csr(), p=d.p))
    gen_s = time.perf_counter() - t0
    # independent problems: each rank (GPU) takes every world-th one, no collective
    from cosmicblup_gb300.ranks import Replicas
    reps = Replicas()
    all_probs, probs = probs, reps.shard(probs)
    out = {}
    for label, prec, workers in [("mixed", MIXED, cfg["workers"]), ("fp64", FP64, cfg["workers"]),
                                 ("mixed_1worker", MIXED, 1)]:
        rc = RemlConfig.default(mode=MODE_EM, precision=prec, max_iter=cfg["max_iter"])
        reps.barrier()
        t0 = time.perf_counter()
        res = batch_reml(probs, rc, workers=workers, device=reps.local_rank)
        wall = reps.max(time.perf_counter() - t0)
        iters = reps.sum(sum(r.iterations for r in res))
        out[label] = {"wall_s": wall, "problems_per_s": len(all_probs) / wall, "reml_iterations": iters,
                      "reml_iter_per_s_incl_setup": iters / wall, "workers": workers,
                      "sum_problem_s": reps.sum(sum(r.seconds for r in res))}
    if reps.rank != 0:
        return
    mtr = run_multi_trait(cfg, reps.local_rank)
    line = {"metric": METRIC, "value": out["mixed"]["reml_iter_per_s_incl_setup"],
            "unit": "REML iter/s (batch, GRM + G^-1 + REML per problem)", "n_gpus": reps.world,
            "scaling": "strong",
            "higher_is_better": True, "dtype": "f32+f64", "data": "synthetic (seeded generator)",
            "config": {"workload": cfg["name"], "problems": cfg["nprob"], "max_iter": cfg["max_iter"],
                       "n_range": [min(p.n for p in all_probs), max(p.n for p in all_probs)],
                       "m_range": [min(p.m for p in all_probs), max(p.m for p in all_probs)],
                       "parallelism": f"problems sharded round robin over {reps.world} GPU(s)"},
            "batch": out, "multi_trait": mtr,
            "mixed_vs_fp64": out["fp64"]["wall_s"] / out["mixed"]["wall_s"],
            "workers_speedup": out["mixed_1worker"]["wall_s"] / out["mixed"]["wall_s"],
            "setup": {"synthetic_data_s": gen_s}}
    print(json.dumps(line))


def run_multi_trait(cfg, device) -> dict:
    """The batch config's dense 3-trait GBLUP: n = 10,000 genotyped animals (m = 20,000
    SNPs), genetic correlations (0.5, -0.3, 0.2), residual correlations 0.1, mean + sex.
    GRM and eigen-bent G^-1 on the device, then MvEigenVce (projection, eigen-EM) and
    the Kronecker multi-trait MME solve, all FP64; host-clock seconds of each call."""
    import ctypes as C
    from cosmicblup_gb300 import Handle, MvEigenVce, MvOptions, invert_psd, solve_multi_trait
    from cosmicblup_gb300._lib import lib, ptr
    from cosmicblup_gb300.synth import simulate_bed, simulate_mt_records
    n, m, seed = cfg["mt_n"], cfg["mt_m"], cfg["seed"] + 7000
    rg = np.array([[1.0, 0.5, -0.3], [0.5, 1.0, 0.2], [-0.3, 0.2, 1.0]])
    sg, se = np.sqrt([0.3, 0.4, 0.5]), np.sqrt([0.7, 0.6, 0.5])
    Vg = rg * np.outer(sg, sg)
    Ve = (np.full((3, 3), 0.1) + 0.9 * np.eye(3)) * np.outer(se, se)
    t0 = time.perf_counter()
    bed, _ = simulate_bed(n, m, seed=seed, p_lo=0.01, miss=0.02)
    rec = simulate_mt_records(bed, n, m, seed=seed + 1, Vg=Vg, Ve=Ve)
    gen_s = time.perf_counter() - t0
    h = Handle(device)
    bedarr = np.frombuffer(bed, dtype=np.uint8)
    s2pq, nval = C.c_double(0), C.c_int64(0)
    t0 = time.perf_counter()
    h.check(lib().cbx_grm_bed(h.raw, ptr(bedarr), bedarr.size, n, m, C.c_float(0.01), 1, 2048, None, None,
                              None, C.byref(s2pq), C.byref(nval)))
    invert_psd(h, None, n, download=False)
    h.sync()
    ginv_s = time.perf_counter() - t0
    v = MvEigenVce(h, MvOptions())
    t0 = time.perf_counter()
    v.prepare(rec["Y"], rec["X"], None)
    v.runNullModel()
    vce_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    sol = solve_multi_trait(h, rec["Y"], rec["X"], v.getVg(), v.getVe(), Ginv=None)
    solve_s = time.perf_counter() - t0
    return {"n": n, "m": m, "traits": 3, "synthetic_data_s": gen_s, "grm_and_ginv_s": ginv_s,
            "vce_s": vce_s, "em_iterations": v.iterations, "converged": v.converged, "solve_s": solve_s,
            "Vg": v.getVg().tolist(), "Ve": v.getVe().tolist(), "Vg_true": Vg.tolist(), "Ve_true": Ve.tolist(),
            "u_abs_max": float(np.abs(sol["u"]).max()),
            "precision": "fp64 (eigen-EM and dense Cholesky of the Kronecker MME, as the reference)"}


def run_geno(h, bed, n, m, seed, hbm_peak, want_host, reps: int = 5) -> dict:
    """SNP-effect back-solve and the genotype products on the resident BED payload.

    snp_effects_ms is end to end (u_g up, G^-1 u on the device, Z^T q, effects down);
    the kernel figures come from CUDA events around each k_geno_zt / k_geno_z launch.
    """
    from cosmicblup_gb300 import DeviceGenotypes
    t0 = time.perf_counter()
    dg = DeviceGenotypes(bed, n, m, h)
    attach_s = time.perf_counter() - t0
    rng = np.random.default_rng(seed + 11)
    u = rng.standard_normal(n)
    w = rng.standard_normal(m)
    dg.snp_effects(u)
    dg.multiply_Z_v(w)
    h.profile(True)
    h.timer_start()
    for _ in range(reps):
        dg.snp_effects(u)
    ms_eff = h.timer_stop() / reps
    zl, zms, zbytes = h.profile_read(3)
    h.profile(True)
    for _ in range(reps):
        dg.multiply_Z_v(w)
    yl, yms, ybytes = h.profile_read(4)
    h.profile(False)
    out = {"workload": f"n={n} samples, m={m} SNPs, one vector", "attach_s": attach_s,
           "snp_effects_ms": ms_eff,
           "k_geno_zt_ms": zms / zl, "k_geno_zt_GBps": zbytes / (zms * 1e-3) / 1e9,
           "k_geno_zt_frac_hbm": zbytes / (zms * 1e-3) / 1e9 / hbm_peak,
           "k_geno_z_ms": yms / yl, "k_geno_z_GBps": ybytes / (yms * 1e-3) / 1e9,
           "elements_per_s_zt": n * m / (zms / zl * 1e-3),
           "note": "exact 64-bit fixed-point sums; integer multiply-issue bound (two 32-bit multiply-adds per code)"}
    if want_host:
        # the C restatement of the reference's multiply_Zt_v loop on a bounded SNP sample,
        # SNP ranges over all host cores as the reference's OpenMP loop, scaled to m
        from oracle.geno import multiply_zt_v_c
        js = min(m, 20000)
        cores = os.cpu_count() or 1
        t0 = time.perf_counter()
        multiply_zt_v_c(bed, n, m, dg.getMeans(), dg.getInvStds(), u, threads=cores, j0=0, j1=js)
        out["cpu_port_zt_ms"] = (time.perf_counter() - t0) * 1e3 * m / js
        out["cpu_port_sample"] = (f"C restatement of the reference's multiply_Zt_v loop on {js} of {m} SNPs, "
                                  f"{cores} threads, scaled to m")
    return out


def run_gpu(args, cfg):
    import ctypes as C
    from cosmicblup_gb300 import AIREML, DeviceMME, Handle, RemlConfig, invert_psd
    from cosmicblup_gb300._lib import lib, pinned, ptr, tune_report
    from cosmicblup_gb300.mme import FP64, MIXED
    from cosmicblup_gb300.vce import MODE_DENSE, MODE_EM, final_solve, reml_gradient

    from cosmicblup_gb300.ranks import Replicas, job_rate
    reps = Replicas()  # host scalars only: the replicas share no data
    world, rank, local = reps.world, reps.rank, reps.local_rank
    hbm_peak, bf16_peak, peak_src = peaks()
    n, m = cfg["n"], cfg["m"]
    G_PROBES = cfg.get("grad_probes", 0) if args.grad_probes is None else args.grad_probes
    dense = bool(cfg.get("dense"))
    mode = MODE_DENSE if dense else MODE_EM
    phases = {}
    h = Handle(local)

    ss = cfg.get("kind") == "ssgblup"
    t0 = time.perf_counter()
    d = build_data(cfg)
    bed, rec, p, rows, q, gmap = d["bed"], d["rec"], d["p"], d["rows"], d["q"], d["gmap"]
    phases["synthetic_data_s"] = time.perf_counter() - t0

    # GRM on the tensor cores
    h.profile(True)
    s2pq, nval = C.c_double(0), C.c_int64(0)
    bedarr = np.frombuffer(bed, dtype=np.uint8)
    t0 = time.perf_counter()
    h.check(lib().cbx_grm_bed(h.raw, ptr(bedarr), bedarr.size, n, m, C.c_float(0.01), 1, 2048, None, None,
                              None, C.byref(s2pq), C.byref(nval)))
    phases["grm_call_s"] = time.perf_counter() - t0
    gl, gms, gops = h.profile_read(2)
    grm = {"n": n, "m_valid": nval.value, "kernel_ms": gms,
           "tops_int8_equivalent": gops / (gms * 1e-3) / 1e12 if gms > 0 else None,
           "frac_of_bf16_peak": gops / (gms * 1e-3) / 1e12 / bf16_peak if gms > 0 else None,
           "note": "2 n^2 m_valid integer ops; exact f16 digit GEMMs on tcgen05 (no int8 MMA on sm_103a)"}

    dm = DeviceMME(h, rec["y"], rec["aid"], rows, p, q)
    want_host = rank == 0 and not args.no_cpu_baseline
    Ainv_h = Gd_h = Ginv_host = None
    if ss:
        # H^-1 blocks on the device: A^-1 (Henderson), A22 by the pedigree
        # recursion, tuneG + blend, eigen-bent Gb^-1 and A22^-1 (FP64)
        from cosmicblup_gb300 import ainv_henderson, ssgblup_qinv
        t0 = time.perf_counter()
        Ainv_h = ainv_henderson(h, d["dam"], d["sire"])
        _, Gd_h = ssgblup_qinv(dm, d["dam"], d["sire"], gmap, G=None, return_blocks=True)
        phases["hinv_setup_s"] = time.perf_counter() - t0
    else:
        # eigen-bent G^-1 (FP64, cuSOLVER syevd + GEMM); host copy for the CPU baseline
        t0 = time.perf_counter()
        Ginv_host = invert_psd(h, None, n, download=want_host)
        phases["g_inverse_s"] = time.perf_counter() - t0
        dm.set_qinv_dense(None)
    fp, fc, fv = rows
    h2d_bytes = rec["y"].nbytes + rec["aid"].nbytes + fp.nbytes + fc.nbytes + fv.nbytes
    if ss:
        # the sparse A^-1 and the genotyped map; the dense H^-1 block stays where the
        # device set-up (GRM, ssgblup_qinv) left it, as G^-1 does for GBLUP
        h2d_bytes += sum(x.nbytes for x in Ainv_h) + gmap.nbytes
    d2h_bytes = 8 * (p + q) + 16 + (16 if G_PROBES else 0)

    def step(r, prec):
        """One REML iteration, then the gradient at its starting point (one call:
        the gradient's probes join the iteration's data + probe block)."""
        if not G_PROBES:
            return r.run_iteration(), None
        info = r.run_iteration(grad_probes=G_PROBES)
        return info, {"grad": info["grad"], "trace": info["grad_trace"], "pcg_iters": info["grad_pcg_iters"]}

    # ---- mixed-precision steps (the headline) ----
    r = AIREML(dm, 0.5, 0.5, RemlConfig.default(mode=mode, precision=MIXED))
    t0 = time.perf_counter()
    for _ in range(args.warmup):
        step(r, MIXED)
    phases["warmup_s"] = time.perf_counter() - t0
    state = (r.var_u, r.var_e)
    h.profile(True)
    clocks = ClockSampler(local)
    clocks.start()
    l0 = h.launches()
    reps.barrier()
    lib().cbx_range_push(b"timed_steps")  # profilers keep this region's kernels
    h.timer_start()
    out = [step(r, MIXED) for _ in range(args.steps)]
    ms_local = h.timer_stop()
    lib().cbx_range_pop()
    launches = h.launches() - l0
    clk = clocks.stop()
    dl, dms, dbytes = h.profile_read(0)
    _, _, ffbytes = h.profile_read(1)
    infos = [o[0] for o in out]
    grads = [o[1] for o in out]
    solves = sum(1 + i["probes"] for i in infos) + sum(G_PROBES + 1 for g in grads if g)
    value, ms = job_rate(args.steps, ms_local, reps)
    solves_per_s, _ = job_rate(solves, ms_local, reps)
    mixed_final = (r.var_u, r.var_e)
    gradient = None
    if G_PROBES:
        gradient = {"probes": G_PROBES,
                    "pcg_iterations_per_step": sum(g["pcg_iters"] for g in grads) / args.steps,
                    "em_probe_solves_reused_per_step": sum(min(i["probes"], G_PROBES) for i in infos) / args.steps,
                    "last": {"grad": list(grads[-1]["grad"]), "trace": grads[-1]["trace"]}}

    # ---- plain FP64 path: the same number of steps from the same start ----
    fp64 = agreement = None
    fp64_steps = args.steps if args.fp64_steps is None else args.fp64_steps
    if fp64_steps > 0 and not dense:
        r64 = AIREML(dm, *state, RemlConfig.default(mode=mode, precision=FP64))
        h.profile(True)
        h.timer_start()
        out64 = [step(r64, FP64) for _ in range(fp64_steps)]
        ms64 = h.timer_stop()
        dl64, dms64, db64 = h.profile_read(1)
        i64 = [o[0] for o in out64]
        g64 = [o[1] for o in out64]
        s64 = sum(1 + i["probes"] for i in i64) + sum(G_PROBES + 1 for g in g64 if g)
        fp64 = {"steps": fp64_steps, "reml_iter_per_s": fp64_steps / (ms64 * 1e-3),
                "pcg_solves_per_s": s64 / (ms64 * 1e-3), "ms_per_step": ms64 / fp64_steps,
                "pcg_iterations_per_step": (sum(i["pcg_iters"] for i in i64)
                                            + sum(g["pcg_iters"] for g in g64 if g)) / fp64_steps,
                "solves_per_step": s64 / fp64_steps,
                "matvecs_per_step": sum(i["matvecs"] for i in i64) / fp64_steps,
                "k_dense_fp64_GBps": db64 / (dms64 * 1e-3) / 1e9 if dms64 > 0 else None,
                "variances": {"var_u": r64.var_u, "var_e": r64.var_e}}
        if fp64_steps == args.steps:
            # the two paths after the same steps from the same start: variance
            # components, final EBVs (each at its own estimates), and the
            # gradient of both at the FP64 estimates.  The forward error of a
            # solve is about cond x relres, so the EBVs are compared from final
            # solves to relres 1e-13, and each path's EBVs at the run's stop
            # (1e-10) are compared with its own tight solve.
            fin = (r64.var_u, r64.var_e)

            def ebv(th, prec, tol):
                return final_solve(dm, *th, solver=1, tol=tol, precision=prec, calc_se=False)["u"]

            def rel(a, b):
                return float(np.abs(a - b).max() / np.abs(b).max())

            sm_t, s64_t = ebv(mixed_final, MIXED, 1e-13), ebv(fin, FP64, 1e-13)
            agreement = {
                "steps": args.steps,
                "max_rel_diff_var": max(abs(mixed_final[0] - fin[0]) / fin[0], abs(mixed_final[1] - fin[1]) / fin[1]),
                "max_rel_diff_ebv": rel(sm_t, s64_t),
                "ebv_note": "final solves to relres 1e-13 at each path's estimates",
                "ebv_forward_error_at_1e-10": {"mixed": rel(ebv(mixed_final, MIXED, 1e-10), sm_t),
                                               "fp64": rel(ebv(fin, FP64, 1e-10), s64_t)},
                "bars": {"var": 1e-6, "ebv": 1e-8}}
            if G_PROBES:
                gm = reml_gradient(dm, *fin, nprobe=G_PROBES, precision=MIXED)["grad"]
                gd = reml_gradient(dm, *fin, nprobe=G_PROBES, precision=FP64)["grad"]
                agreement["max_rel_diff_grad"] = float(np.abs(gm - gd).max() / np.abs(gd).max())

    # ---- end to end through the C ABI from host buffers ----
    # A REML run from the same start as the timed steps above, in which every
    # iteration uploads the records, the design (and A^-1) again, rebuilds the
    # MME and runs the iteration (with its gradient), its solution coming back.
    # The handle keeps the last solutions of the previous MME as the starting
    # points of the next one's solves (cbx_mme_keep_warm), as the reference keeps
    # last_solution across iterations; the first iteration starts cold.  The same
    # warm-up iterations run untimed, so the timed iterations are the same ones
    # as the device-timed steps'.
    e2e_steps = max(1, min(args.steps, 3))
    host_inputs = [rec["y"], rec["aid"], fp, fc, fv] + (list(Ainv_h) + [gmap] if ss else [])
    e2e_pcg_iters = 0

    def e2e_step(theta):
        dm2 = DeviceMME(h, rec["y"], rec["aid"], (fp, fc, fv), p, q)
        if ss:
            dm2.set_qinv_split(*Ainv_h, gmap=gmap)
        else:
            dm2.set_qinv_dense(None)
        r2 = AIREML(dm2, *theta, RemlConfig.default(mode=mode, precision=MIXED, max_iter=1))
        if G_PROBES:
            # the iteration and its gradient in one call; the data solve comes back
            info = r2.run_iteration(grad_probes=G_PROBES, solution=True)
            its = info["pcg_iters"] + info["grad_pcg_iters"]
        else:
            r2.solve()
            its = 0
        return (r2.var_u, r2.var_e), its, dm2

    # the step's host inputs sit in page-locked memory (registered once, outside the
    # timed region); every step copies them to the device again
    with pinned(*host_inputs):
        h.keep_warm(False)
        theta = (0.5, 0.5)
        for i in range(args.warmup):
            theta, _, dm2 = e2e_step(theta)
            h.keep_warm(True)
        reps.barrier()
        h.timer_start()
        for _ in range(e2e_steps):
            theta, its, dm2 = e2e_step(theta)
            e2e_pcg_iters += its
        e2e_rate, _ = job_rate(e2e_steps, h.timer_stop(), reps)
        h.keep_warm(False)
    e2e = {"value": e2e_rate, "unit": UNIT,
           "h2d_bytes_per_step": int(h2d_bytes), "d2h_bytes_per_step": int(d2h_bytes),
           "steps": e2e_steps, "pcg_iterations_per_step": e2e_pcg_iters / e2e_steps if G_PROBES else None}

    # ---- genotype products: SNP-effect back-solve effect = Z^T G^-1 u / total 2pq ----
    geno = None
    if not ss:
        geno = run_geno(h, bed, n, m, cfg["seed"], hbm_peak, want_host)

    # ---- CPU baseline: the reference's algorithm on this operator, bounded sample ----
    cpu = None
    if want_host:
        from oracle.mme import MME, build_fixed_design, sparse_data_part
        _, orows, _ = build_fixed_design(rec["cats"])
        cores = os.cpu_count()
        if dense:
            from oracle.reml import AIREML as OracleREML
            o = OracleREML(MME(rec["y"], rec["aid"], orows, p, q), Ginv_host, *state)
            o.dense_exact_step()
            t0 = time.perf_counter()
            o.dense_exact_step()
            c = time.perf_counter() - t0
            cpu = {"value": 1.0 / c, "unit": UNIT, "cores": cores, "kind": "port",
                   "sample": f"one oracle dense exact AI-REML step on this problem (numpy/BLAS, {cores} threads)"}
        else:
            from oracle.rng import rademacher
            WtW, W = sparse_data_part(rec["aid"], orows, p, q)
            lam = state[1] / state[0]
            iters = 10 if n >= 10000 else 50
            if ss:
                import scipy.sparse as sp
                ap, ac, av = Ainv_h
                c = cpu_pcg_iteration_cost(WtW, Gd_h, p, lam, iters, Ainv=sp.csr_matrix((av, ac, ap), shape=(q, q)),
                                           gmap=gmap)
            else:
                c = cpu_pcg_iteration_cost(WtW, Ginv_host, p, lam, iters)
            # PCG iterations per solve of the reference's algorithm on this operator,
            # counted in this run: the data right-hand side and two probes, each a
            # single-RHS FP64 PCG from zero to relres 1e-10 (the GPU's FP64 path runs
            # the same iterations as the oracle's PCG, in seconds instead of minutes)
            B = [W.T @ rec["y"]]
            for z in rademacher(42, q, 2):
                b = np.zeros(p + q)
                b[p:] = z
                B.append(b)
            its = [int(dm2.pcg_solve(lam, b, precision=FP64)[1][0]) for b in B]
            per_solve = float(np.mean(its)) + 1.0
            em_probes = sum(i["probes"] for i in infos) / args.steps
            nsolve = solves_per_step(cfg, em_probes)
            work = nsolve * per_solve
            cpu = {"value": 1.0 / (c * work), "unit": UNIT, "cores": cores, "kind": "port",
                   "sample": (f"oracle FP64 PCG, {iters} iterations on this operator (numpy/BLAS, {cores} "
                              f"threads) = {c * 1e3:.1f} ms per iteration; x {work:.0f} single-RHS operator "
                              f"applications per step = {nsolve:.0f} solves x {per_solve:.0f} (PCG iterations "
                              f"per solve from zero counted in this run: data {its[0]}, probes {its[1]}, "
                              f"{its[2]})")}

    if rank != 0:
        return
    ach = dbytes / (dms * 1e-3) / 1e9 if dms > 0 else None
    block_mb = 4.0 * n * n / 1e6
    l2_note = (f"inputs larger than L2 ({block_mb / 1e3:.2f} GB FP32 dense block read per PCG iteration)"
               if block_mb > 129.0 else
               f"the {block_mb:.0f} MB FP32 dense block fits in L2 (no flush between iterations): "
               f"a cache-resident figure, not an HBM one")
    if dense:
        l2_note = f"dense exact step on {p + q}-order FP64 matrices (32 MB each); cache-resident"
    step_desc = ("one dense exact AI-REML step (FP64 Cholesky, P, AI traces, logL-checked halving)" if dense else
                 "one EM+Hutchinson AI-REML iteration (data solve + adaptive probe solves, relres 1e-10)"
                 + (f", then the REML gradient at its starting point from {G_PROBES} probes (cbx_reml_iterate_grad: "
                    f"the gradient's first probes, up to 79, solved in the iteration's data + probe block, the "
                    f"iteration's estimator using only the probes its stopping rule selects)" if G_PROBES else ""))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if dense else "f32+f64",
        "data": "synthetic (seeded generator with the workload's shapes)",
        "config": {"workload": cfg["name"], "n_animals": q, "n_genotyped": n, "n_snps": m,
                   "fixed_levels": cfg["levels"], "step": step_desc,
                   "precision": ("fp64" if dense else "mixed: FP32 PCG bulk + FP64 refinement on the true residual"),
                   "genotypes": "gene-dropped through the pedigree" if ss else "HWE, independent samples",
                   "l2": l2_note,
                   "parallelism": f"replicas x{world}"},
        "pcg_solves_per_s": solves_per_s,
        "pcg_iterations_per_step": (sum(i["pcg_iters"] for i in infos)
                                    + sum(g["pcg_iters"] for g in grads if g)) / args.steps,
        "probes_per_step": sum(i["probes"] for i in infos) / args.steps,
        "gradient": gradient,
        "fp64": fp64,
        "mixed_vs_fp64": (value / world) / fp64["reml_iter_per_s"] if fp64 else None,
        "agreement": agreement,
        "grm": grm,
        "snp_backsolve": geno,
        "setup": phases,
        "clocks": clk,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm",
                     "kernel": (("k_dense_tf32<128, 80>" if G_PROBES else "k_dense_tf32<64>")
                                + " (tcgen05 3xTF32, dense H^-1 / G^-1 block x the populated columns of the "
                                  "solver block)"),
                     "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                     "frac": (ach / hbm_peak) if ach else None,
                     "traffic": TRAFFIC_BYTES.get((n, 128 if G_PROBES else 64)),
                     "peak_source": peak_src, "launches": dl, "avg_launch_ms": dms / dl if dl else None,
                     "step_dense_bytes_GBps": (dbytes + ffbytes) / (ms_local * 1e-3) / 1e9,
                     "step_hbm_frac": (dbytes + ffbytes) / (ms_local * 1e-3) / 1e9 / hbm_peak,
                     "step_note": "the step's dense-block bytes (FP32 products and FP64-accurate "
                                  "refinement products) over the whole step time; sparse and vector "
                                  "traffic not counted"},
        "cpu_baseline": cpu,
        "variances": {"var_u": r.var_u, "var_e": r.var_e},
        "autotune": tune_report(),
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="cbx", choices=["cbx", "reference"])
    ap.add_argument("--config", default="c3", choices=sorted(CONFIGS))
    ap.add_argument("--fp64-steps", type=int, default=None,
                    help="FP64 comparison steps (default: --steps)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--grad-probes", type=int, default=None,
                    help="probes of the gradient in each step (default: the config's)")
    args = ap.parse_args()
    cfg = CONFIGS[args.config]
    if args.impl == "reference":
        run_reference(args, cfg)
    elif cfg.get("kind") == "batch":
        run_batch(args, cfg)
    else:
        run_gpu(args, cfg)


if __name__ == "__main__":
    main()
