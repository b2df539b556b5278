"""Placement throughput benchmark (query placements/s) on one GB300.

Workload: dna_1k -- the batched-FP32 configuration: Yule tree of 1,000 taxa
(branch lengths ~ Exp(0.05)), DNA GTR+G4, 1,500-site alignment, 10,000 queries
of masked length U[100, 1500] with 2% substitution noise and 1% internal gaps,
pplacer default placement preferences (keep-at-most 7, max-strikes 6,
strike-box 3, max-pitches 40), seeded synthetic data (seed 1001).

A step is the whole placement phase for all queries (stage-1 ranking of every
edge, baseball stage-2 branch-length optimisation, final refinement at 1e-5,
like_weight_ratio), after the reference-tree precompute, as pplacer times it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--optimizer newton|brent] [--queries Q]

value: placements/s with queries and GLVs already resident in HBM, timed with
       CUDA events on the engine's stream; the GLV arrays (3 x 192 MB) exceed
       the 129 MB L2, so no L2 flush is needed between steps.
e2e:   placements/s through pgb_place_batch (the C ABI call a caller makes)
       with the query rows in page-locked host memory (pgb_host_alloc),
       uploaded, placed and the placements copied back every step.

--workload aa_500 | cat_5k | dna_2k runs the other configurations through the
same line (20-state + G4 on the tensor-core kernel, GTR + CAT 20 and the long
nucleotide queries on the warp kernel); the roofline block names the kernel
that ran.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


# measured constants of the stage-2 roofline (see the roofline block below)
DRAM_BYTES_PER_SITE_EVAL = 78.63  # k_place_warp (eigenbasis form on packed FP32 pairs, 12 warps/SM) on dna_1k: 24.004 GB DRAM read + write / 305.3 M site evaluations
# FFMA + FMUL per site and rate with derivatives (the kernel's arithmetic):
# six 4x4 matrix-vector products (96) + the six sums (52) in the matrix form;
# 2 x 3 coordinate scalings + 6 x 12 column FMAs (78) + 52 in the eigenbasis form
# CAT in the eigenbasis: 6 x 3 scalings + 6 x 12 column FMAs (90) + 52
FMA_OPS_PER_SITE_RATE = {"matrix": 148, "eigenbasis": 130, "CAT eigenbasis": 142}
N_SM = 152
SM_MAX_HZ = 2.07e9


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--optimizer", default="newton", choices=["newton", "brent"])
    ap.add_argument("--qng-sample", type=int, default=1000,
                    help="queries of the posterior-probability leg computed as the reference does (pp_rule 1)")
    ap.add_argument("--pp-steps", type=int, default=1,
                    help="untimed-region comparison: placement steps with posterior probabilities")
    ap.add_argument("--brent-steps", type=int, default=2,
                    help="untimed-region comparison: placement steps with the Brent replica")
    ap.add_argument("--queries", type=int, default=None)
    ap.add_argument("--workload", default="dna_1k")
    ap.add_argument("--cpu-sample", type=int, default=512, help="queries in the CPU-baseline sample")
    ap.add_argument("--dropin-sample", type=int, default=3,
                    help="queries placed by pplacer's flow over the plain per-call drop-in (untimed region)")
    ap.add_argument("--batch", type=int, default=0,
                    help="device batch of the end-to-end pgb_place_batch calls (0: automatic)")
    ap.add_argument("--precompute-steps", type=int, default=2,
                    help="untimed-region comparison: reference-tree precomputes (and CAT category refinements)")
    return ap.parse_args()


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return rank, world, local, dist
    return rank, world, local, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        med = sorted(sm)[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# The nucleotide Gamma warp forms by the engine's tuning value (smem_windows
# of a warp bin): 0 matrices in registers, 1-3 the eigenbasis form
WARP_FORM_WARPS = {0: 8, 1: 8, 2: 12, 3: 16, 4: 12, 5: 16}


def warp_form(w, tune):
    """'matrix' or 'eigenbasis' for the nucleotide warp kernel; None otherwise."""
    if w.site_cats is not None or w.K != 4 or set(int(v) for v in tune[0]) != {32}:
        return None
    return "eigenbasis" if int(tune[1][0]) >= 1 else "matrix"


def stage2_kernel(w, tune):
    """The trial kernel that ran stage 2 + refinement for this workload and tuning."""
    th = set(int(v) for v in tune[0])
    if w.prefs.get("max_strikes") == 0 and len(w.query_seqs) < 2 * 8 * N_SM and th == {32}:
        return ("k_trials_warp (every edge of every query: all stage-2 trials in one launch, one warp each; "
                "then the refinement trials)")
    if th == {32}:
        return "k_place_warp (stage 2 + refinement, whole queries, one warp each%s)" % (
            ", per-site categories, %s form" % {0: "matrix", 1: "eigenbasis", 2: "eigenbasis on packed FP32 pairs"}[
                int(tune[1][0])]
            if w.site_cats is not None else
            ", %s form%s, %d warps per SM" % (warp_form(w, tune), " on packed FP32 pairs" if int(tune[1][0]) >= 4 else "",
                                             WARP_FORM_WARPS[int(tune[1][0])]))
    if th == {1}:
        return ("k_place_tc (stage 2 + refinement, whole queries, one 128-thread team each, two teams per CTA, "
                "tcgen05 evolves)")
    if len(th) == 1:
        return "k_place_cta (stage 2 + refinement, whole queries, one CTA of %d threads each)" % th.pop()
    return "k_trials (stage 2 + refinement in baseball rounds, CTA per trial, %s threads)" % "/".join(
        str(t) for t in sorted(th))


def load_peaks():
    try:
        with open(MEASURED_PEAKS) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_bf16_peak():
    """Dense bf16 TFLOP/s of this GPU (burst: the stage-1 GEMMs run for well
    under a second)."""
    try:
        with open(MEASURED_PEAKS) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def cpu_baseline(w, n_sample, prefs_kw):
    """The oracle (FP64 CPU restatement of pplacer's path, with the reference's
    own linear_c.c arithmetic) on a bounded sample, all host threads."""
    from oracle import oracle as O
    O.build(with_ref=True)
    n = min(n_sample, len(w.query_seqs))
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ref = O.Reference(O.Model(w.exch, w.statd, w.rates, w.site_cats), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    t_pre = time.perf_counter() - t0
    t0 = time.perf_counter()
    ref.place(w.query_seqs[:n], O.make_prefs(**prefs_kw), n_threads=threads)
    dt = time.perf_counter() - t0
    return n / dt, threads, n, dt, t_pre


def cpu_refine_pass(w):
    """One of the oracle's category passes of the CAT site-category
    refinement (gcat_model.ml:387-419: the whole tree's per-site likelihood
    with every site in one category), one thread; the refinement runs one
    per category."""
    import numpy as np
    from oracle import oracle as O
    t0 = time.perf_counter()
    cat = np.zeros(w.n_sites, dtype=np.int32)
    O.Reference(O.Model(w.exch, w.statd, w.rates, cat), w.parent, w.bl, w.leaf_row, w.ref_seqs).root_site_loglike()
    return time.perf_counter() - t0


def run_reference(args):
    rank, world, local, dist = dist_setup(args.gpus)
    if rank != 0:
        return
    from pplacer_gb300 import synth
    w = synth.make_workload(args.workload, n_queries=args.queries)
    prefs_kw = dict(w.prefs)
    from oracle import oracle as O
    O.build(with_ref=True)
    threads = os.cpu_count() or 1
    ref = O.Reference(O.Model(w.exch, w.statd, w.rates, w.site_cats), w.parent, w.bl, w.leaf_row, w.ref_seqs)
    n = min(args.cpu_sample // 2, len(w.query_seqs))
    for i in range(args.warmup):
        ref.place(w.query_seqs[:max(8, n // 8)], O.make_prefs(**prefs_kw), n_threads=threads)
    t0 = time.perf_counter()
    for i in range(args.steps):
        lo = (i * n) % len(w.query_seqs)
        ref.place((w.query_seqs + w.query_seqs)[lo:lo + n], O.make_prefs(**prefs_kw), n_threads=threads)
    dt = time.perf_counter() - t0
    v = n * args.steps / dt
    line = {"metric": "query placements/s", "value": v, "unit": "placements/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "queries_per_step": n, "taxa": (w.n_nodes + 1) // 2,
                       "sites": w.n_sites},
            "cpu_baseline": {"value": v, "unit": "placements/s", "cores": threads, "kind": "port",
                             "sample": "%d queries of %s per step" % (n, args.workload)},
            "e2e": {"value": v, "unit": "placements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def plain_dropin_brent(eng, w, prefs, n_sample, brent_res):
    """pplacer's own per-query flow over the plain drop-in, measured: the
    Linear externals (linear.ml:13-89) replaced one for one by the pgb_* C
    ABI, each call copying its operands in and its result out, the GLVs on
    the host as the OCaml side keeps them; process_query (core.ml:113-409)
    with its alternating GSL Brent searches (dropin_flow.place_query).
    n_sample queries are placed and timed by wall clock; their best edges
    are compared with the batched Brent replica's."""
    import numpy as np
    from pplacer_gb300 import dropin_flow as DF
    m = eng.model
    model = DF.Model(m.statd, m.x, m.lam, m.xit, m.rates)
    nodes = range(len(w.parent))
    darr, parr, snodes = {}, {}, {}
    for i in nodes:
        if w.parent[i] < 0:
            continue
        darr[i] = DF.Glv(*eng.get_glv(0, i))
        parr[i] = DF.Glv(*eng.get_glv(1, i))
        snodes[i] = DF.Glv(*eng.get_glv(2, i))
    edges = [i for i in nodes if w.parent[i] >= 0]
    pf = {k: getattr(prefs, k) for k in ("start_pend", "max_pend", "initial_tolerance", "max_pitches", "max_strikes",
                                         "strike_box", "keep_at_most", "keep_factor")}
    t0 = time.perf_counter()
    calls, agree, placed = 0, 0, []
    for q in range(n_sample):
        res, n = DF.place_query(model, w.query_seqs[q], darr, parr, snodes, w.bl, edges, pf)
        calls += n
        placed.append(res)
        agree += int(bool(res) and bool(brent_res[q]) and res[0][0] == brent_res[q][0][0])
    dt = time.perf_counter() - t0
    return {"value": n_sample / dt, "unit": "placements/s",
            "method": "measured: pplacer's per-query flow over the pgb_* drop-in calls, wall clock",
            "sample_queries": n_sample, "seconds": dt, "brent_evals_per_query": calls / n_sample,
            "best_edge_agrees_with_batched_brent": "%d/%d" % (agree, n_sample)}


def run_ours(args):
    rank, world, local, dist = dist_setup(args.gpus)
    import numpy as np
    from pplacer_gb300 import build as B
    B.build()
    from pplacer_gb300 import engine as E
    from pplacer_gb300 import lib as L
    from pplacer_gb300 import synth
    w = synth.make_workload(args.workload, n_queries=args.queries)
    Q, S = len(w.query_seqs), w.n_sites
    eng = E.engine_for_workload(w)
    prefs = E.default_prefs(optimizer=1 if args.optimizer == "newton" else 0, **w.prefs)
    lib = L.load()
    # ---- device-resident value ----
    eng.load_queries(w.query_seqs)
    tune = eng.autotune(prefs)
    for _ in range(args.warmup):
        eng.run(prefs)
    barrier(dist)
    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.start()
    n0 = lib.pgb_kernel_launch_count()
    ms_steps, phase = [], np.zeros(6)
    counts = np.zeros(8)
    for _ in range(args.steps):
        eng.run(prefs)
        ms, cnt = eng.timings()
        ms_steps.append(ms[5])
        phase += ms
        counts += cnt
    launches = lib.pgb_kernel_launch_count() - n0
    barrier(dist)
    clocks = sampler.stop() if sampler else None
    t_dev = max_over_ranks(dist, sum(ms_steps) / 1e3)
    value = Q * world * args.steps / t_dev
    # ---- the reference's optimiser (GSL Brent replica) on the same kernel path ----
    brent = None
    if args.optimizer == "newton" and args.brent_steps > 0:
        bprefs = E.default_prefs(optimizer=0, **w.prefs)
        eng.run(bprefs)
        bms, bev, btr = 0.0, 0.0, 0.0
        for _ in range(args.brent_steps):
            eng.run(bprefs)
            ms, cnt = eng.timings()
            bms += ms[5]
            bev += cnt[2]
            btr += cnt[1]
        brent = {"value": Q * args.brent_steps / (bms / 1e3), "unit": "placements/s",
                 "evals_per_trial": bev / btr, "evals_per_query": bev / (args.brent_steps * Q),
                 "steps": args.brent_steps}
        if args.dropin_sample > 0 and w.site_cats is None:
            bres, _ = eng.fetch()
            brent["plain_dropin"] = plain_dropin_brent(eng, w, bprefs, min(args.dropin_sample, Q), bres)
            brent["newton_over_plain_dropin"] = value / brent["plain_dropin"]["value"]
        brent["newton_over_batched_brent"] = value / brent["value"]
    # ---- posterior probabilities (-p, default exponential prior) on the same path ----
    pp = None
    if args.optimizer == "newton" and args.pp_steps > 0:
        pprefs = E.default_prefs(optimizer=1, calc_pp=1, **w.prefs)
        eng.run(pprefs)
        pms, pev = 0.0, 0.0
        for _ in range(args.pp_steps):
            eng.run(pprefs)
            ms, cnt = eng.timings()
            pms += ms[5]
            pev += cnt[2]
        pp = {"value": Q * args.pp_steps / (pms / 1e3), "unit": "placements/s",
              "evals_per_step": pev / args.pp_steps, "steps": args.pp_steps,
              "quadrature": "Gauss-Legendre panels around the optimum (pp_rule 0)"}
        # the reference's own computation of the marginal likelihood (pp_rule
        # 1: find_upper_limit's Brent search, nested QNG to pp_rel_err, ETOL
        # retries), on the CTA kernels that carry it; a bounded sample of the
        # queries (it evaluates ~20x more points per placement)
        nq = min(Q, args.qng_sample)
        eng.load_queries(w.query_seqs[:nq])
        qprefs = E.default_prefs(optimizer=1, calc_pp=1, pp_rule=1, **w.prefs)
        eng.run(qprefs)
        eng.run(qprefs)
        ms, cnt = eng.timings()
        pp["reference_qng"] = {"value": nq / (ms[5] / 1e3), "unit": "placements/s", "evals_per_step": cnt[2],
                               "steps": 1, "queries": nq}
        eng.load_queries(w.query_seqs)
    # ---- end to end through pgb_place_batch: the query rows in, the
    # placements out, both in page-locked host memory (pgb_host_alloc) ----
    kam = prefs.keep_at_most
    hb_in = L.HostBuffer(Q * S)
    hb_in.array(np.uint8, Q * S)[:] = np.frombuffer("".join(w.query_seqs).encode(), dtype=np.uint8)
    hb_out = L.HostBuffer(Q * kam * C.sizeof(L.Placement) + 8 * Q)
    out_p = hb_out.address
    n_out_p = out_p + Q * kam * C.sizeof(L.Placement)
    qst_p = n_out_p + 4 * Q
    lib.pgb_place_batch(eng.h, C.byref(prefs), Q, hb_in.address, args.batch, out_p, n_out_p, qst_p)
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        L.check(lib.pgb_place_batch(eng.h, C.byref(prefs), Q, hb_in.address, args.batch, out_p, n_out_p, qst_p),
                "pgb_place_batch")
    t_e2e = max_over_ranks(dist, time.perf_counter() - t0)
    assert int(hb_out.array(np.int32, Q * kam * C.sizeof(L.Placement) // 4 + Q)[-Q:].sum()) > 0  # placements came back
    hb_in.close()
    hb_out.close()
    e2e = Q * world * args.steps / t_e2e
    # ---- the reference-tree precompute (like_stree.ml:43-110: distal and
    # proximal GLVs, exponent pulls, supernodes) and, for CAT models, the
    # site-category refinement (gcat_model.ml:387-419), by wall clock through
    # the C ABI: host preparation, uploads, kernels and the final
    # synchronisation; last, as the refinement replaces the categories ----
    pre = None
    if args.precompute_steps > 0:
        tp = []
        for _ in range(args.precompute_steps):
            t0 = time.perf_counter()
            eng.precompute(w.leaf_row, w.ref_seqs)
            tp.append(time.perf_counter() - t0)
        pre = {"gpu_ms": 1e3 * min(tp), "steps": args.precompute_steps}
        if w.site_cats is not None:
            tr = []
            for _ in range(args.precompute_steps):
                t0 = time.perf_counter()
                eng.refine_categories(w.leaf_row, w.ref_seqs)
                tr.append(time.perf_counter() - t0)
            pre["refine_categories_gpu_ms"] = 1e3 * min(tr)
    if rank != 0:
        return
    # ---- roofline of the dominant kernel ----
    # Stage 2 + refinement run as one launch of the whole-query warp kernel
    # (k_place_warp) per step; its duration is the engine's stage-2 event
    # interval.  Algorithmic bytes per site evaluation of a fused forward +
    # adjoint evaluation: the distal and proximal GLV windows, FP32 entries
    # of every rate plus the int32 exponent, 2 * (4 * R * K + 4), and the
    # query's character code, 1 -- 137 B for DNA G4.
    R, K = len(w.rates) if w.site_cats is None else 1, w.K
    bytes_per_site_eval = 2 * (4 * R * K + 4) + 1
    site_evals = counts[3]
    t_trials = phase[3] / 1e3 / args.steps
    peak, peak_kind = load_peaks()
    achieved = bytes_per_site_eval * site_evals / args.steps / t_trials / 1e9 if t_trials > 0 else 0.0
    # DRAM traffic per site evaluation from one ncu capture of k_place_warp on
    # this workload (dram__bytes_read.sum + dram__bytes_write.sum over the
    # launch's site evaluations, full-size dna_1k capture)
    traffic = (DRAM_BYTES_PER_SITE_EVAL * site_evals / args.steps
               if args.workload == "dna_1k" and DRAM_BYTES_PER_SITE_EVAL else None)
    # the binding unit is instruction issue on the FP32 pipe: FMA-pipe lane
    # operations per site evaluation of the form that ran (per rate, with
    # derivatives), against 128 lanes per SM; CAT runs the matrix arithmetic
    # on its one plane, the 20-state tensor-core form has no such count
    cat_warp = w.site_cats is not None and set(int(v) for v in tune[0]) == {32}
    form = warp_form(w, tune) or ((("CAT eigenbasis" if int(tune[1][0]) >= 1 else "matrix")) if cat_warp else None)
    fp32_ops = (FMA_OPS_PER_SITE_RATE[form] * R * site_evals / args.steps / t_trials
                if form and t_trials > 0 else None)
    fp32_peak = 128 * N_SM * SM_MAX_HZ
    # Stage 1 (the masked_logdot score of every (query, edge) pair): the
    # tcgen05 kernel k_s1_mma contracts [edges x queries] over K = 3 x prim x
    # Sc (the bf16 hi / mid / lo terms of the log-likelihood tables, one-hot
    # in the query's code) + 2 x Sc (the exponent digits), Sc = sites padded
    # to 32; counted on the unpadded edges and queries, timed alone
    prim = 4 if K == 4 else 20
    n_edges = int(np.sum(np.asarray(w.parent) >= 0))
    Sc = (S + 31) // 32 * 32
    s1_flops = 2.0 * n_edges * Q * (3 * prim * Sc + 2 * Sc)
    t_s1 = phase[0] / 1e3 / args.steps
    bf16_peak, bf16_kind = load_bf16_peak()
    s1_tflops = s1_flops / t_s1 / 1e12 if t_s1 > 0 else 0.0
    cpu_v, cpu_threads, cpu_n, cpu_dt, cpu_pre = cpu_baseline(w, args.cpu_sample, dict(w.prefs))
    if pre is not None:
        pre["cpu_ms"] = 1e3 * cpu_pre
        pre["cpu"] = "the oracle's FP64 precompute (reference construction), one thread"
        if "refine_categories_gpu_ms" in pre:
            pre["refine_categories_cpu_ms"] = 1e3 * cpu_refine_pass(w) * len(w.rates)
            pre["refine_categories_cpu"] = ("one category pass of the oracle's refinement, one thread, "
                                            "times the %d categories" % len(w.rates))
    line = {
        "metric": "query placements/s", "value": value, "unit": "placements/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": args.workload, "taxa": (w.n_nodes + 1) // 2, "sites": S, "queries": Q,
                   "model": ("GTR+CAT%d" % (int(np.max(w.site_cats)) + 1) if w.site_cats is not None
                             else ("20-state+G%d" if K == 20 else "GTR+G%d") % len(w.rates)),
                   "optimizer": args.optimizer, "keep_at_most": prefs.keep_at_most,
                   "max_strikes": prefs.max_strikes,
                   "trial_tuning": {"threads": [int(v) for v in tune[0]], "smem_windows": [int(v) for v in tune[1]]},
                   "l2": "GLV arrays 3x%.0f MB exceed L2, no flush" %
                   (w.n_nodes * S * R * K * 4 / 1e6), "seed": w.seed},
        "edge_evals": {"stage1_pairs_per_s": counts[0] / (phase[2] / 1e3),
                       "stage2_evals_per_s": counts[2] / (phase[3] / 1e3),
                       "trials_per_step": counts[1] / args.steps,
                       "stage2_trials_launched": counts[4] / args.steps,
                       "stage2_trials_consumed": counts[5] / args.steps,
                       "refine_trials": counts[6] / args.steps, "rounds": counts[7] / args.steps,
                       "phase_ms": {"stage1_table": phase[1] / args.steps, "stage1_rank": phase[2] / args.steps, "stage1_contraction": phase[0] / args.steps,
                                    "stage2": phase[3] / args.steps, "refine_out": phase[4] / args.steps}},
        "roofline": {"kernel": stage2_kernel(w, tune), "bound": "hbm", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "traffic_unit": "bytes per launch",
                     "traffic_source": ("ncu capture of the full-size dna_1k launch (dram__bytes_read.sum + "
                                        "dram__bytes_write.sum), per site evaluation, scaled to this launch"
                                        if traffic is not None else None),
                     "algorithmic_bytes_per_site_eval": bytes_per_site_eval,
                     "peak_source": peak_kind,
                     "fp32_pipe": ({"achieved": fp32_ops, "peak": fp32_peak, "unit": "FMA-pipe lane ops/s",
                                    "frac": fp32_ops / fp32_peak, "ops_per_site_rate": FMA_OPS_PER_SITE_RATE[form],
                                    "form": form, "peak_source": "nominal: 128 lanes x 152 SMs x 2070 MHz"}
                                   if fp32_ops is not None else None),
                     "stage1": {"kernel": "k_s1_mma (hand-written tcgen05: TMA bf16 tables, one-hot query tiles "
                                          "built in shared memory, TMEM accumulators)", "bound": "tensor",
                                "achieved": s1_tflops, "peak": bf16_peak, "unit": "TFLOP/s",
                                "frac": s1_tflops / bf16_peak, "peak_source": bf16_kind,
                                "flops_per_step": s1_flops, "ms_per_step": 1e3 * t_s1,
                                "note": "the contraction alone; the ranking (k_rank_warp) is in phase_ms.stage1_rank"}},
        "cpu_baseline": {"value": cpu_v, "unit": "placements/s", "cores": cpu_threads, "kind": "port",
                         "sample": "%d queries of %s (%.1f s)" % (cpu_n, args.workload, cpu_dt)},
        "e2e": {"value": e2e, "unit": "placements/s", "h2d_bytes_per_step": Q * S,
                "d2h_bytes_per_step": Q * kam * C.sizeof(L.Placement) + 8 * Q,
                "device_batch": args.batch if args.batch else "automatic"},
        "brent_replica": brent,
        "with_posterior_probabilities": pp,
        "tree_precompute": pre,
        "newton_evals_per_trial": counts[2] / counts[1] if counts[1] else None,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
