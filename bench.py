#!/usr/bin/env python
"""Benchmark: exact 10-NN queries/s at n = 10,000,000, d = 128 on GB300.

Workload (default, the configuration the headline metric is quoted on):
  database  n = 10,000,000 rows, d = 128, integer features drawn i.i.d. from a
            geometric distribution with mean 20 clipped to 255 (stored as
            float32), from the engine's counter-based generator, seed 3;
  queries   m = 10,000 rows from the same distribution (independent stream);
  search    exact 10-NN under squared L2, results sorted by (distance, id),
            1,024 representatives (measured on GB300 at 512 / 1,024 / 4,096:
            239k / 245k / 211k queries/s for the headline form, about 7,100
            for the plain form at each count).
One step = one exact query call for all m queries with the index and the
queries resident in HBM.  The 5.12 GB database is far larger than the 129 MB
L2, so no flush is needed between steps.

Forms timed on the same index (all exact, identical ids):
  plain    FP32 list search on the CUDA cores (the plain RBC)
  tensor   BF16 tcgen05 list search + FP32 rerank (certified)
  learned  tensor form whose probe round follows the learned router, trained
           on the GPU beforehand on queries labelled by the RBC itself
The headline `value` is the learned+BF16 form, as the metric names it.

`--workload c5` measures the learned-router configuration instead (n =
4,194,304, 2,000-component Gaussian mixture with sigma ~ U[0.02, 0.1],
4,096 representatives, router trained on 1,000,000 queries, 100,000 test
queries) and reports probe recall and lists searched per query.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

Multi-GPU runs are independent replicas (queries need no exchange): one
process per GPU under torchrun, each with its own index, value = all ranks'
queries / the slowest rank's time.  `--impl reference` times the reference's
CPU brute-force path on this host's cores instead.
"""
import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "randomballcover-gpu_gb300")
sys.path.insert(0, PKG)

METRIC = "exact 10-NN queries/s, n=10M d=128, learned+BF16 vs plain FP32 RBC, same GPU"
UNIT = "queries/s"

WORKLOADS = {
    # kind, seed, n, m, d, k, reps, ncomp, sigma_lo, sigma_hi, train queries, router epochs, forms
    "c1": dict(kind=0, seed=1, n=65_536, m=8_192, d=16, k=1, reps=256, ncomp=1, slo=0.0, shi=0.0,
               train=0, epochs=0, forms="oneshot,tensor,plain",
               metric="exact 1-NN queries/s, n=65,536 d=16 uniform, plain FP32 RBC",
               desc="i.i.d. uniform [0,1)"),
    "c2": dict(kind=1, seed=2, n=1_048_576, m=100_000, d=128, k=32, reps=1024, ncomp=1000, slo=0.05, shi=0.05,
               train=0, epochs=0, forms="oneshot,tensor,plain",
               metric="exact 32-NN queries/s, n=1,048,576 d=128 mixture, plain FP32 RBC",
               desc="1,000-component Gaussian mixture, sigma 0.05"),
    "c3": dict(kind=2, seed=3, n=10_000_000, m=10_000, d=128, k=10, reps=1024, ncomp=1, slo=0.0, shi=0.0,
               train=100_000, epochs=2, forms="plain,tensor,learned", metric=METRIC,
               desc="geometric(mean 20) integer features"),
    "c4": dict(kind=1, seed=4, instances=64, n_lo=10_000, n_hi=2_000_000, dims=(32, 64, 128), ks=(1, 10, 32),
               comp_lo=100, comp_hi=1000, slo=0.05, shi=0.05, forms="fp32,tensor",
               metric="exact k-NN queries/s over 64 batched heterogeneous RBC instances (one graph)",
               desc="64 instances, n log-uniform in [1e4, 2e6], d in {32, 64, 128}, k in {1, 10, 32}, m = n/100"),
    "c5": dict(kind=1, seed=5, n=4_194_304, m=100_000, d=128, k=10, reps=4096, ncomp=2000, slo=0.02, shi=0.1,
               train=1_000_000, epochs=3, forms="plain,tensor,learned",
               metric="exact 10-NN queries/s, n=4,194,304 d=128 mixture, learned router + BF16 vs plain FP32 RBC",
               desc="2,000-component Gaussian mixture, sigma ~ U[0.02, 0.1]"),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="c3", choices=sorted(WORKLOADS))
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--m", type=int, default=None)
    ap.add_argument("--reps", type=int, default=None)
    ap.add_argument("--train", type=int, default=None)
    ap.add_argument("--cpu-queries-per-thread", type=int, default=6)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-side", action="store_true",
                    help="skip the c2 side measurements (k = 128 and the double-precision variant)")
    ap.add_argument("--router-probes", type=int, default=2,
                    help="lists the learned form probes from the router (the tuner then tries 1 and 2; "
                         "0: none, the distance head plans instead)")
    ap.add_argument("--forms", default=None,
                    help="forms to time; the last one listed is the headline (default: per workload)")
    ap.add_argument("--item-rows", type=int, default=0,
                    help="longest row run of one work item (rbc_set_tuning; 0: the index's default)")
    ap.add_argument("--tc-tuning", default=None, metavar="PROBES,ROWS[,CAP]",
                    help="fixed tensor-form knobs instead of timing them (profiling runs): probed lists, FP32 "
                         "prefix rows, and the probe cap (rows; 0 or absent: none)")
    a = ap.parse_args()
    w = dict(WORKLOADS[a.workload])
    for key in ("n", "m", "reps", "train"):
        if getattr(a, key) is not None:
            w[key] = getattr(a, key)
    if a.forms is None:
        a.forms = w["forms"]
    a.w = w
    return a


def config(a, form):
    w = a.w
    if a.workload == "c4":
        return {"workload": f"c4: {w['desc']}, squared L2", "instances": w["instances"], "form": form,
                "l2_flush": "inputs larger than L2 (GBs of databases vs 129 MB L2); no flush between steps"}
    return {"workload": f"{a.workload}: exact {w['k']}-NN, n={w['n']:,} d={w['d']} {w['desc']}, "
                        f"m={w['m']:,} queries, squared L2",
            "n": w["n"], "d": w["d"], "m": w["m"], "k": w["k"], "num_reps": w["reps"], "form": form,
            "l2_flush": "inputs larger than L2 (the database is GBs vs 129 MB L2); no flush between steps"}


# ------------------------------------------------------------------ clocks
CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class ClockSampler:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={CLOCK_FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        sm = [float(r[1]) for r in rows if re.match(r"^[\d.]+$", r[1])]
        mx = [float(r[2]) for r in rows if re.match(r"^[\d.]+$", r[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------ helpers
def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(v, dist, device):
    """The largest of every rank's v (v itself without a process group)."""
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(per_rank_units, steps, world, slowest_ms):
    """Whole-job rate of N independent replicas: every rank's units over the
    slowest rank's time (weak scaling: each rank holds the full per-GPU work)."""
    return world * per_rank_units * steps / (slowest_ms / 1000.0)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        j = json.load(open(p))
        return j["hbm_gbs"], j["bf16_tflops"], j.get("bf16_tflops_sustained"), "measured"
    return 6800.0, 1900.0, 1700.0, "fallback"


def committed_traffic(kernel, workload=None):
    """Per-launch DRAM bytes of a kernel at a workload's default size, from the
    committed ncu summary (a line `traffic_bytes_per_launch_<workload>: B`),
    if any."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_traffic.md")
    if not workload or not os.path.exists(path):
        return None
    m = re.search(rf"traffic_bytes_per_launch_{workload}:\s*([\d.eE+]+)", open(path).read())
    return float(m.group(1)) if m else None


def fp64_error(X, Q, ids, dists, sample=512):
    """Largest |d - d64| / d64 of the returned squared L2 distances over a
    query sample, d64 recomputed in float64 from the same rows."""
    import torch
    S = min(sample, Q.shape[0])
    sel = torch.linspace(0, Q.shape[0] - 1, S, device=Q.device).long()
    I = ids[sel].long()
    valid = I >= 0  # unfilled slots hold 0xFFFFFFFF
    rows = X[I.clamp(min=0)].double()
    d64 = ((rows - Q[sel].double()[:, None, :]) ** 2).sum(-1)
    d32 = dists[sel].double()
    pos = valid & (d64 > 0)
    if bool((valid & (d64 == 0) & (d32 != 0)).any().item()):
        return float("inf")
    return float(((d32 - d64).abs() / d64)[pos].max().item()) if bool(pos.any().item()) else 0.0


# ------------------------------------------------------------------ CPU baselines
def host_matrix(w, stream, rows, threads):
    """Rows of the synthetic matrix generated on the host by the CPU recipe."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build(with_ref=False)
    X = np.empty((rows, w["d"]), np.float32)
    T = oracle.geometric_table()
    chunk = (rows + threads - 1) // threads

    def fill(t):
        r0 = t * chunk
        r1 = min(rows, r0 + chunk)
        if r1 > r0:
            X[r0:r1] = oracle.synth(w["kind"], w["seed"], stream, r1 - r0, w["d"], r0=r0, ncomp=w["ncomp"],
                                    sigma_lo=w["slo"], sigma_hi=w["shi"], table=T)

    ths = [threading.Thread(target=fill, args=(t,)) for t in range(threads)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    return X


def cpu_knn_timed(X, Qs, k, threads):
    """Time the reference's CPU path on Qs: its own bruteCPU (1-NN, compiled from
    the reference sources) when that build is present, else the oracle's
    restatement of the same distance loop with (dist, id) k-NN selection.
    Returns (seconds, kind, description, answer); answer is (ids, dists) of
    the k-NN, or (1-NN ids as one column, None) from bruteCPU."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    if oracle.ref_available():
        out = np.empty(Qs.shape[0], np.uint32)
        shards = np.array_split(np.arange(Qs.shape[0]), threads)

        def run(ix):
            if len(ix):
                q = np.ascontiguousarray(Qs[ix])
                o = np.empty(len(ix), np.uint32)
                oracle.ref_brute_cpu_raw(X, X.shape[0], X.shape[1], q, len(ix), o)
                out[ix] = o

        t0 = time.perf_counter()
        ths = [threading.Thread(target=run, args=(ix,)) for ix in shards]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        return time.perf_counter() - t0, "reference", "bruteCPU (brute.cu:91-112), 1-NN", (out[:, None], None)
    t0 = time.perf_counter()
    ans = oracle.knn(X, Qs, k, threads=threads)
    return time.perf_counter() - t0, "port", f"oracle restatement of distVec/bruteCPU, {k}-NN", ans


PARITY_RTOL = 1e-6  # distance tolerance (relative); ids must be equal bit for bit


def compare_answers(got_ids, got_d, want):
    """(ids equal, distances equal bit for bit, distances within PARITY_RTOL)
    of a GPU answer against the oracle's (k columns, or bruteCPU's 1-NN column)."""
    want_ids, want_d = want
    g = np.ascontiguousarray(got_ids).view(np.uint32)
    if want_d is None:
        return bool((g[:, 0] == want_ids[:, 0]).all()), None, None
    gd = np.asarray(got_d, np.float32)
    ids_eq = bool((g == want_ids).all())
    bits = bool((gd.view(np.uint32) == want_d.view(np.uint32)).all())
    tol = bool((np.abs(gd.astype(np.float64) - want_d) <= PARITY_RTOL * np.abs(want_d.astype(np.float64))).all())
    return ids_eq, bits, tol


def parity_report(results, forms, sel, want, extra_rows=None, extra_want=None):
    """Every listed form's answers on the sampled queries `sel` against the
    oracle's; extra_rows / extra_want: more queries (the tensor forms'
    FP32-fallback queries) checked the same way."""
    out = {"queries": int(len(sel)), "forms": list(forms), "ids_equal": True, "dists_equal": True,
           "dists_within_rtol": True, "rtol": PARITY_RTOL, "per_form": {}}
    for f in forms:
        r = results[f]
        ids_eq, bits, tol = compare_answers(r["ids"][sel].cpu().numpy(), r["dists"][sel].cpu().numpy(), want)
        row = {"ids_equal": ids_eq, "dists_equal": bits, "dists_within_rtol": tol}
        if extra_rows is not None and len(extra_rows):
            e_ids, e_bits, e_tol = compare_answers(r["ids"][extra_rows].cpu().numpy(),
                                                   r["dists"][extra_rows].cpu().numpy(), extra_want)
            row["fallback_queries"] = {"queries": int(len(extra_rows)), "ids_equal": e_ids, "dists_equal": e_bits}
            ids_eq, bits, tol = ids_eq and e_ids, bits and e_bits, tol and e_tol
        out["per_form"][f] = row
        out["ids_equal"] &= ids_eq
        out["dists_equal"] = None if bits is None else (out["dists_equal"] and bits)
        out["dists_within_rtol"] = None if tol is None else (out["dists_within_rtol"] and tol)
    out["fallback_queries_checked"] = int(len(extra_rows)) if extra_rows is not None else 0
    return out


def parity_failed(p):
    return p is not None and (not p["ids_equal"] or p["dists_within_rtol"] is False)


# ------------------------------------------------------------------ reference arm
def run_reference(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    w = a.w
    if a.workload == "c4":  # the largest instance of the batch stands for the workload
        specs = batch_instances(w)
        i = max(range(len(specs)), key=lambda j: specs[j][0])
        n, d, k, m, ncomp, _ = specs[i]
        w = dict(w, seed=w["seed"] * 1000 + i, n=n, d=d, k=k, m=m, ncomp=ncomp)
        a.w = dict(w, reps=0)
    threads = os.cpu_count() or 1
    X = host_matrix(w, 0, w["n"], threads)
    Q = host_matrix(w, 1, min(w["m"], 4096), threads)
    per_step = 2 * threads

    def step(i):
        lo = (i * per_step) % Q.shape[0]
        qs = np.ascontiguousarray(Q[lo:lo + per_step])
        if qs.shape[0] < per_step:
            qs = np.ascontiguousarray(Q[:per_step])
        return cpu_knn_timed(X, qs, w["k"], threads)

    for i in range(a.warmup):
        step(i)
    total = 0.0
    kind = desc = None
    for i in range(a.steps):
        t, kind, desc, _ = step(a.warmup + i)
        total += t
    value = per_step * a.steps / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1000 * total / a.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (counter-based generator, CPU recipe)", "config": config(a, "reference CPU brute force"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": f"{per_step} queries per step over the full {w['n']:,}-row database; {desc}"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ engine arm
def run_engine(a):
    import torch
    import pyrbc

    w = a.w
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    def maxall(v):
        return max_over_ranks(v, dist, "cuda")

    stream = torch.cuda.current_stream()
    synth = dict(ncomp=w["ncomp"], sigma_lo=w["slo"], sigma_hi=w["shi"])
    X = pyrbc.synth(w["kind"], w["seed"], 0, w["n"], w["d"], **synth)
    Q = pyrbc.synth(w["kind"], w["seed"], 1, w["m"], w["d"], **synth)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    forms = [f for f in a.forms.split(",") if f]
    head = forms[-1]
    flags = pyrbc.BUILD_PARTITION | pyrbc.BUILD_BF16 | (pyrbc.BUILD_ONESHOT if "oneshot" in forms else 0)
    idx = pyrbc.Index(X, w["reps"], s=w["reps"], seed=w["seed"], flags=flags)
    build_s = time.perf_counter() - t0
    info = idx.info()
    k, m = w["k"], w["m"]

    # the learned router: trained on the GPU on queries the RBC labels
    router_info = None
    if "learned" in forms:
        # the router's two heads, trained on labels the RBC produces: the list
        # owning each training query's nearest neighbour, and its k-th
        # distance over its nearest representative's
        Qtr = pyrbc.synth(w["kind"], w["seed"], 2, w["train"], w["d"], **synth)
        t0 = time.perf_counter()
        labels, tdist, tnear = idx.router_labels(Qtr, k)
        torch.cuda.synchronize()
        label_s = time.perf_counter() - t0
        router = pyrbc.Router(w["d"], 512, w["reps"], seed=w["seed"], distance_head=True)
        t0 = time.perf_counter()
        loss = router.train_with_distance(Qtr, labels, tdist, tnear, epochs=w["epochs"], batch=1024, lr=2e-3,
                                          seed=w["seed"])
        torch.cuda.synchronize()
        train_s = time.perf_counter() - t0
        del Qtr, labels, tdist, tnear
        test_labels, true_d, near_d = idx.router_labels(Q, k)
        top1 = router.logits(Q).argmax(1)
        ratio = (router.predict_distance(Q, near_d) / true_d).float()
        mu, sg, margin = router.distance_params()
        router_info = {"train_queries": w["train"], "epochs": w["epochs"], "label_s": label_s, "train_s": train_s,
                       "final_loss": loss, "probe_recall_top1": (top1 == test_labels.long()).float().mean().item(),
                       "distance_head": {"median_predicted_over_true": ratio.median().item(),
                                         "share_below_true": (ratio < 1).float().mean().item(),
                                         "margin_sigma_units": margin, "log_ratio_sigma": sg},
                       "architecture": f"MLP {w['d']}->512->512->{w['reps']} (+1 distance output) GELU, "
                                       "BF16 weights, FP32 accumulate"}
        # the router's picks join the probe round (the tuner chooses one or two
        # and whether the nearest representatives' lists come too); with
        # --router-probes 0 the predicted k-th distance plans the search instead
        idx.set_router(router, probes=a.router_probes)

    modes = {"plain": pyrbc.QUERY_EXACT, "tensor": pyrbc.QUERY_EXACT_TC, "oneshot": pyrbc.QUERY_ONESHOT,
             "learned": pyrbc.QUERY_EXACT_TC | pyrbc.QUERY_ROUTED, "learned_plain": pyrbc.QUERY_EXACT | pyrbc.QUERY_ROUTED}
    if a.item_rows:
        idx.set_tuning(0, a.item_rows)
    idx.set_profiling(True)
    ids = torch.empty((m, k), dtype=torch.int32, device="cuda")
    dists = torch.empty((m, k), dtype=torch.float32, device="cuda")

    # the tensor form's knobs are tuned per form on queries drawn apart from
    # the timed ones (same distribution), outside the timed region, as many as
    # one timed call holds (up to 100,000): the best probe round depends on
    # how many queries share a probed list (c5 tuned on 20,000 chose the FP32
    # probe round, 1.757M queries/s; on 100,000 the tensor one, 1.83M)
    Qtune = pyrbc.synth(w["kind"], w["seed"], 3, min(m, 100_000), w["d"], **synth)
    tuning = {}

    def timed(mode, steps, warmup, sample_clocks=False):
        if mode & pyrbc.QUERY_EXACT_TC and k <= 32:
            if a.tc_tuning:
                knobs = [int(v) for v in a.tc_tuning.split(",")]
                idx.set_tc_tuning(*knobs[:2])
                idx.set_tc_probe_cap(knobs[2] if len(knobs) > 2 else 0)
            else:
                idx.autotune_tc(Qtune, k, mode)
            inf = idx.info()
            p_, r_ = idx.tc_tuning()
            tuning[mode] = ["router picks only" if p_ == pyrbc.TC_ROUTER_ONLY else p_,
                            "no FP32 prefix" if r_ == pyrbc.TC_PREFIX_NONE else r_]
            tuning[mode] += [f"probe cap {inf['tc_probe_cap']} rows"] if inf["tc_probe_cap"] else []
            tuning[mode] += ["plain FP32 search chosen"] if inf["tc_plain"] else []
            if mode & pyrbc.QUERY_ROUTED:
                tuning[mode].append("router not consulted (the tuner measured the nearest lists alone faster)"
                                    if inf["tc_unrouted"] else f"router picks {inf['router_picks']}")
        for _ in range(warmup):
            idx.query(Q, k, mode=mode, out=(ids, dists))
        barrier()
        clocks = ClockSampler(local) if sample_clocks else None
        if clocks:
            clocks.start()
        l0 = pyrbc.kernel_launches()
        acc = {"search_ms": 0.0, "search_launches": 0, "point_pairs": 0, "lists": 0, "fallback": 0,
               "pruned_ms": 0.0, "pruned_launches": 0, "pruned_pairs": 0}
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            idx.query(Q, k, mode=mode, out=(ids, dists))
            p = idx.profile()
            st = idx.stats()
            acc["search_ms"] += p["search_ms"]
            acc["search_launches"] += p["search_launches"]
            for key in ("pruned_ms", "pruned_launches", "pruned_pairs"):
                acc[key] += p[key]
            acc["point_pairs"] += st["point_pairs"]
            acc["lists"] += st["lists_probed"]
            acc["fallback"] += st["fallback_queries"]
        ev1.record(stream)
        barrier()
        acc["launches"] = pyrbc.kernel_launches() - l0
        acc["clocks"] = clocks.stop() if clocks else None
        acc["ms"] = maxall(ev0.elapsed_time(ev1))
        acc["steps"] = steps
        acc["value"] = replica_rate(m, steps, world, acc["ms"])
        acc["ids"] = ids.clone()
        acc["dists"] = dists.clone()
        acc["fallback_ids"] = idx.fallback_queries() if mode & pyrbc.QUERY_EXACT_TC else np.empty(0, np.uint32)
        acc["fp64"] = fp64_error(X, Q, ids, dists)
        return acc

    results = {}
    for f in forms:
        if f == head:
            results[f] = timed(modes[f], a.steps, a.warmup, sample_clocks=True)
        else:
            results[f] = timed(modes[f], min(a.steps, 3), 1)
    res = results[head]
    exact_forms = [f for f in results if f != "oneshot"]
    same = all(bool((results[f]["ids"] == results[exact_forms[-1]]["ids"]).all().item()) for f in exact_forms)
    oneshot_recall = None
    if "oneshot" in results and exact_forms:
        # the reference's one-shot algorithm is approximate: share of the exact k-NN it returns
        ex, os_ = results[exact_forms[-1]]["ids"].long(), results["oneshot"]["ids"].long()
        hit = (os_[:, :, None] == ex[:, None, :]).any(2).float().mean().item()
        oneshot_recall = hit
    range_count = None
    if a.workload in ("c1", "c2"):
        # brute-force range count (bruteRangeCount) of a query sample, ranges = the k-th exact distance
        nq = min(m, 2048)
        ranges = results[exact_forms[-1]]["dists"][:nq, k - 1].contiguous() if exact_forms else None
        if ranges is not None:
            pyrbc.range_count(X, Q[:nq], ranges)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            cnt = pyrbc.range_count(X, Q[:nq], ranges)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            range_count = {"queries": nq, "ms": dt * 1e3, "pairs_per_s": nq * w["n"] / dt,
                           "all_counts_at_least_k_minus_1": bool((cnt >= k - 1).all().item())}
    side = side_measurements(a, idx, X, Q, results, exact_forms) if (a.workload == "c2" and not a.no_side) else None
    clk, value, ms, launches = res["clocks"], res["value"], res["ms"], res["launches"]

    # end to end through the host API: pinned host queries in, results out
    Qh = Q.cpu().pin_memory()
    ih = torch.empty((m, k), dtype=torch.int32).pin_memory()
    dh = torch.empty((m, k), dtype=torch.float32).pin_memory()
    idx.query_host(Qh.numpy(), k, mode=modes[head], out=(ih.numpy().view(np.uint32), dh.numpy()))
    barrier()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        idx.query_host(Qh.numpy(), k, mode=modes[head], out=(ih.numpy().view(np.uint32), dh.numpy()))
    e2e_s = maxall(time.perf_counter() - t0)
    e2e = {"value": world * m * a.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(m * w["d"] * 4),
           "d2h_bytes_per_step": int(m * k * 8)}

    # roofline of the dominant kernel; algorithmic work = 2 d flops per
    # (query, database row) pair the search evaluates
    hbm, bf16, bf16_sus, src = peaks()
    flops_per_launch = res["point_pairs"] * 2 * w["d"] / max(res["search_launches"], 1)
    avg_launch_s = res["search_ms"] / max(res["search_launches"], 1) / 1000.0
    achieved = flops_per_launch / avg_launch_s / 1e12 if avg_launch_s > 0 else 0.0
    sm_mhz = (clk or {}).get("sm_mhz") or 1920.0
    head_plain = head == "plain" or (modes[head] & pyrbc.QUERY_EXACT_TC and idx.info()["tc_plain"])
    kernel = "search_kernel" if head_plain else "tc_search_kernel"
    roofline = {"bound": "tensor", "achieved": achieved, "peak": bf16, "unit": "TFLOP/s",
                "frac": achieved / bf16, "traffic": committed_traffic(kernel, a.workload if a.n is None and a.m is None else None), "kernel": kernel,
                "peak_source": f"{src} bf16 dense burst (MEASURED_PEAKS.json)",
                "flops_per_launch": flops_per_launch, "avg_launch_ms": avg_launch_s * 1e3}
    if not head_plain and res["pruned_launches"] and res["pruned_launches"] < res["search_launches"]:
        # the tensor form launches two instances of its list search per
        # call: the pruned round (two query tiles per B tile, the dominant
        # launch) and the probe round's large lists (one query tile); the
        # roofline is the pruned round's, both together are listed beside it
        pl = res["pruned_launches"]
        p_flops = res["pruned_pairs"] * 2 * w["d"] / pl
        p_s = res["pruned_ms"] / pl / 1000.0
        o_l = res["search_launches"] - pl
        o_s = (res["search_ms"] - res["pruned_ms"]) / max(o_l, 1) / 1000.0
        o_flops = (res["point_pairs"] - res["pruned_pairs"]) * 2 * w["d"] / max(o_l, 1)
        all_launches = {k_: roofline.pop(k_) for k_ in ("achieved", "frac", "flops_per_launch", "avg_launch_ms")}
        roofline.update({"achieved": p_flops / p_s / 1e12, "frac": p_flops / p_s / 1e12 / bf16,
                         "kernel": f"tc_search_kernel<MT={1 if idx.info()['tc_format'] else 2}> (pruned round)",
                         "flops_per_launch": p_flops,
                         "avg_launch_ms": p_s * 1e3,
                         "probe_round_launch": {"kernel": "tc_search_kernel<MT=1> (probe round, large lists)",
                                                "avg_launch_ms": o_s * 1e3, "flops_per_launch": o_flops,
                                                "achieved": o_flops / o_s / 1e12 if o_s > 0 else 0.0},
                         "all_tensor_launches": all_launches})
    if head_plain:
        fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
        roofline["fp32_core"] = {"achieved_tflops": achieved, "peak_tflops": fp32_peak, "frac": achieved / fp32_peak,
                                 "note": "difference form costs sub+mul+add per pair-dim, 2 flops counted"}

    cpu = None
    parity = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        # the CPU baseline's answers double as the full-size parity check:
        # queries spread evenly over the batch, every exact form compared
        # with them bit for bit, plus every query a tensor form sent to its
        # FP32 fallback (up to 256), whose oracle answers are computed here
        threads = os.cpu_count() or 1
        nq = min(m, a.cpu_queries_per_thread * threads)
        sel = np.unique(np.linspace(0, m - 1, nq).round().astype(np.int64))
        Xh = X.cpu().numpy()
        Qs = Q[torch.from_numpy(sel).cuda()].cpu().numpy()
        t, kind, desc, ans = cpu_knn_timed(Xh, Qs, k, threads)
        cpu = {"value": len(sel) / t, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": f"{len(sel)} of the {m:,} queries (evenly spaced) over the full {w['n']:,}-row database; "
                         f"{desc}"}
        fb = np.unique(np.concatenate([results[f]["fallback_ids"] for f in exact_forms] or [np.empty(0)]))
        fb = fb.astype(np.int64)[:256]
        fb_want = None
        if len(fb):
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle
            fb_want = oracle.knn(Xh, Q[torch.from_numpy(fb).cuda()].cpu().numpy(), k, threads=threads)
        parity = parity_report(results, exact_forms, sel, ans, fb if len(fb) else None, fb_want)
        parity["oracle"] = kind

    if rank == 0:
        names = {"plain": "plain FP32 exact RBC", "tensor": "exact RBC, BF16 tcgen05 list search + FP32 rerank",
                 "oneshot": "the reference's one-shot RBC (approximate)",
                 "learned": "exact RBC, learned router (its picks in the probe round) + BF16 tcgen05 list search "
                            "+ FP32 rerank",
                 "learned_plain": "exact RBC, learned router + FP32 list search"}
        extra = {"build_s": build_s, "min_list": info["min_list"], "max_list": info["max_list"],
                 "tc_format": ["bf16", "fp16_split"][info["tc_format"]], "same_ids_all_exact_forms": same,
                 "router": router_info, "oneshot_recall": oneshot_recall, "range_count": range_count, "forms": {},
                 "side": side}
        for f, r in results.items():
            extra["forms"][f] = {"value": r["value"], "ms_per_step": r["ms"] / r["steps"],
                                 "tc_probes_and_probe_rows": tuning.get(modes[f]),
                                 "lists_per_query": r["lists"] / (m * r["steps"]),
                                 "pairs_per_query": r["point_pairs"] / (m * r["steps"]),
                                 "fallback_queries_per_step": r["fallback"] / r["steps"],
                                 "max_rel_dist_error_vs_fp64": r["fp64"]}
        if "plain" in results:
            extra["speedup_vs_plain_fp32"] = value / results["plain"]["value"]
        line = {"metric": w["metric"], "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32" if head == "plain" else "bf16+f32",
                "data": "synthetic (counter-based generator on the GPU)",
                "config": dict(config(a, names[head]), parallelism=f"replicas{world}"),
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
                "clocks": clk, "parity": parity, "extra": extra}
        print(json.dumps(line), flush=True)
    idx.close()
    if dist:
        dist.destroy_process_group()
    if parity_failed(parity):
        sys.exit("parity: GPU answers differ from the oracle's")


def side_measurements(a, idx, X, Q, results, exact_forms):
    """Paths beyond the headline, on a query sample of the same workload:
    k = 128 (FP32 lists of 128 entries) and the double-precision variant
    (FP32 shortlists reranked in double, certified), plus the double brute
    force's own rate (range count in double: every pair in FP64)."""
    import torch
    import pyrbc
    w = a.w
    k, ms = w["k"], min(w["m"], 20_000)
    Qs = Q[:ms].contiguous()

    def clock(fn):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    out = {"queries": ms}
    (i128, d128), dt = clock(lambda: idx.query(Qs, 128))
    st = idx.stats()
    ref = results[exact_forms[-1]]["ids"][:ms] if exact_forms else None
    out["k128"] = {"value": ms / dt, "unit": UNIT, "pairs_per_query": st["point_pairs"] / ms,
                   "first_k_equal_k_query": bool((i128[:, :k] == ref).all().item()) if ref is not None else None,
                   "sorted": bool((d128[:, 1:] >= d128[:, :-1]).all().item())}
    t0 = time.perf_counter()
    idx64 = pyrbc.Index(X.double(), w["reps"], seed=w["seed"])
    torch.cuda.synchronize()
    build64 = time.perf_counter() - t0
    Q64 = Qs.double()
    (i64, d64), dt = clock(lambda: idx64.query(Q64, k))
    st = idx64.stats()
    out["f64"] = {"value": ms / dt, "unit": UNIT, "k": k, "build_s": build64,
                  "queries_searched_in_double": st["fallback_queries"],
                  "ids_equal_fp32_answer": (i64 == ref).float().mean().item() if ref is not None else None}
    idx64.close()
    nq = 256
    r = d64[:nq, k - 1].contiguous()
    X64 = X.double()
    _, dt = clock(lambda: pyrbc.range_count(X64, Q64[:nq], r))
    out["f64_scan"] = {"queries": nq, "pairs_per_s": nq * w["n"] / dt,
                       "fp64_gflops": nq * w["n"] * 3 * w["d"] / dt / 1e9,
                       "note": "double brute force (range count): sub, mul, add per pair-dim, all FP64"}
    del X64
    return out


def batch_instances(w):
    """The heterogeneous instances of the batched workload: (n, d, k, m, ncomp, reps)."""
    rng = np.random.default_rng(w["seed"])
    out = []
    for _ in range(w["instances"]):
        n = int(round(np.exp(rng.uniform(np.log(w["n_lo"]), np.log(w["n_hi"])))))
        d = int(rng.choice(w["dims"]))
        k = int(rng.choice(w["ks"]))
        ncomp = int(rng.integers(w["comp_lo"], w["comp_hi"] + 1))
        reps = int(min(4096, max(64, round(2 * np.sqrt(n)))))
        out.append((n, d, k, max(1, n // 100), ncomp, reps))
    return out


def run_batch(a):
    """64 independent (database, query set) instances answered by one captured
    graph per step (rbc_batch), in two variants: the FP32 search (one
    persistent launch per round over every instance) and the tensor form
    (BF16 / FP16 hi-lo operands on tcgen05, uncertified queries searched
    again on the device inside the graph).  Each is compared with answering
    the instances one by one."""
    import torch
    import pyrbc

    w = a.w
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    stream = torch.cuda.current_stream()
    forms = [f for f in a.forms.split(",") if f]
    head = forms[-1]
    modes = {"fp32": pyrbc.QUERY_EXACT, "tensor": pyrbc.QUERY_EXACT_TC}
    specs = batch_instances(w)
    inst = []
    t0 = time.perf_counter()
    for i, (n, d, k, m, ncomp, reps) in enumerate(specs):
        syn = dict(ncomp=ncomp, sigma_lo=w["slo"], sigma_hi=w["shi"])
        X = pyrbc.synth(w["kind"], w["seed"] * 1000 + i, 0, n, d, **syn)
        Q = pyrbc.synth(w["kind"], w["seed"] * 1000 + i, 1, m, d, **syn)
        idx = pyrbc.Index(X, reps, seed=i, flags=pyrbc.BUILD_PARTITION | pyrbc.BUILD_BF16)
        idx.autotune(Q, k)
        if "tensor" in forms:
            idx.autotune_tc(Q, k)
        inst.append({"X": X, "Q": Q, "idx": idx, "k": k, "m": m, "n": n, "d": d})
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    total_m = sum(r["m"] for r in inst)
    hbm, bf16, bf16_sus, src = peaks()
    res = {}
    for f in forms:
        mode = modes[f]
        # one by one (the same exact query per instance), for comparison and the pair counts
        pairs = flops = fallbacks = 0
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        seq = []
        for r in inst:
            seq.append(r["idx"].query(r["Q"], r["k"], mode=mode))
            st = r["idx"].stats()
            pairs += st["point_pairs"]
            flops += st["point_pairs"] * 2 * r["d"]
            fallbacks += st["fallback_queries"]
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(a.steps):
            for r in inst:
                r["idx"].query(r["Q"], r["k"], mode=mode)
        ev1.record(stream)
        torch.cuda.synchronize()
        seq_ms = ev0.elapsed_time(ev1) / a.steps
        batch = pyrbc.Batch()
        outs = [batch.add(r["idx"], r["Q"], r["k"], mode=mode) for r in inst]
        for _ in range(a.warmup):
            batch.run()
        torch.cuda.synchronize()
        same = all(bool((o[0] == s_[0]).all().item()) and bool((o[1] == s_[1]).all().item())
                   for o, s_ in zip(outs, seq))
        fp64 = max(fp64_error(r["X"], r["Q"], o[0], o[1], sample=64) for r, o in zip(inst, outs))
        clocks = ClockSampler(local) if f == head else None
        if clocks:
            clocks.start()
        l0 = pyrbc.kernel_launches()
        # an NVTX range around the timed steps (a profiler can keep to it)
        torch.cuda.nvtx.range_push(f"batch_{f}")
        ev0.record(stream)
        for _ in range(a.steps):
            batch.run()
        ev1.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        clk = clocks.stop() if clocks else None
        launches = pyrbc.kernel_launches() - l0
        ms = max_over_ranks(ev0.elapsed_time(ev1), dist, "cuda")
        sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
        achieved = flops / (ms / a.steps / 1000.0) / 1e12
        if f == "fp32":
            fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
            roof = {"bound": "fp32 pipe", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                    "frac": achieved / fp32_peak, "traffic": committed_traffic("search_kernel_batch"),
                    "kernel": "search_kernel (whole graph step)",
                    "peak_source": f"FP32 pipe: 152 SMs x 128 lanes x 2 flops x {sm_mhz:.0f} MHz (no measured "
                                   "FP32 peak; the difference form issues 3 instructions per 2 flops counted)",
                    "note": "achieved = evaluated (query, row) pairs x 2d over the whole graph step"}
        else:
            roof = {"bound": "tensor", "achieved": achieved, "peak": bf16, "unit": "TFLOP/s",
                    "frac": achieved / bf16, "traffic": committed_traffic("tc_search_kernel_batch"),
                    "kernel": "tc_search_kernel (whole graph step)",
                    "peak_source": f"{src} bf16 dense burst (MEASURED_PEAKS.json)",
                    "note": "achieved = evaluated (query, row) pairs x 2d over the whole graph step; the FP16 "
                            "hi/lo operands take 3 MMAs per pair"}
        res[f] = {"batch": batch, "outs": outs, "ms": ms, "value": replica_rate(total_m, a.steps, world, ms),
                  "launches": launches, "clocks": clk, "roofline": roof, "seq_ms": seq_ms, "pairs": pairs,
                  "same": same, "fp64": fp64, "fallbacks": fallbacks}

    h = res[head]
    batch, outs, ms = h["batch"], h["outs"], h["ms"]
    # end to end: pinned host queries copied in, results copied out, every step
    hq = [r["Q"].cpu().pin_memory() for r in inst]
    hi = [torch.empty_like(o[0], device="cpu").pin_memory() for o in outs]
    hd = [torch.empty_like(o[1], device="cpu").pin_memory() for o in outs]
    h2d = sum(q.numel() * 4 for q in hq)
    d2h = sum(o[0].numel() * 8 for o in outs)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        for r, q in zip(inst, hq):
            r["Q"].copy_(q, non_blocking=True)
        batch.run()
        for o, i_, d_ in zip(outs, hi, hd):
            i_.copy_(o[0], non_blocking=True)
            d_.copy_(o[1], non_blocking=True)
        torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": world * total_m * a.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h)}
    cpu = None
    parity = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        threads = os.cpu_count() or 1
        r = max(inst, key=lambda z: z["n"])
        nq = min(r["m"], 2 * threads)
        t, kind, desc, _ = cpu_knn_timed(r["X"].cpu().numpy(), r["Q"][:nq].cpu().numpy(), r["k"], threads)
        cpu = {"value": nq / t, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": f"{nq} queries of the largest instance (n={r['n']:,}, d={r['d']}); {desc}"}
        # parity: 4 queries of every instance (first, last, two between)
        # against the oracle, every variant's batched answers bit for bit
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        parity = {"queries": 0, "instances": len(inst), "forms": forms, "ids_equal": True, "dists_equal": True,
                  "dists_within_rtol": True, "rtol": PARITY_RTOL}
        for j, r in enumerate(inst):
            sel = np.unique(np.linspace(0, r["m"] - 1, min(4, r["m"])).round().astype(np.int64))
            tsel = torch.from_numpy(sel).cuda()
            want = oracle.knn(r["X"].cpu().numpy(), r["Q"][tsel].cpu().numpy(), r["k"], threads=threads)
            parity["queries"] += len(sel)
            for f in forms:
                o = res[f]["outs"][j]
                ids_eq, bits, tol = compare_answers(o[0][tsel].cpu().numpy(), o[1][tsel].cpu().numpy(), want)
                parity["ids_equal"] &= ids_eq
                parity["dists_equal"] &= bits
                parity["dists_within_rtol"] &= tol
        parity["oracle"] = "port"
    if rank == 0:
        extra = {"build_and_tune_s": build_s, "queries_per_step": total_m, "forms": {},
                 "instances": [{"n": r["n"], "d": r["d"], "k": r["k"], "m": r["m"]} for r in inst]}
        for f, r_ in res.items():
            extra["forms"][f] = {"value": r_["value"], "ms_per_step": r_["ms"] / a.steps,
                                 "launches_per_step": r_["launches"] / a.steps, "pairs_per_step": r_["pairs"],
                                 "one_by_one_ms_per_step": r_["seq_ms"],
                                 "one_by_one_value": world * total_m / (r_["seq_ms"] / 1000.0),
                                 "batched_speedup": r_["seq_ms"] / (r_["ms"] / a.steps),
                                 "same_ids_as_one_by_one": r_["same"], "max_rel_dist_error_vs_fp64": r_["fp64"],
                                 "uncertified_queries_per_step": r_["fallbacks"],
                                 "roofline": r_["roofline"]}
        names = {"fp32": "batched exact RBC, FP32 list search, CUDA graph",
                 "tensor": "batched exact RBC, tcgen05 list search + FP32 rerank, CUDA graph"}
        line = {"metric": w["metric"], "value": h["value"], "unit": UNIT, "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32" if head == "fp32" else "bf16/fp16+f32",
                "data": "synthetic (counter-based generator on the GPU)",
                "config": dict(config(a, names[head]), parallelism=f"replicas{world}"),
                "roofline": h["roofline"], "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(h["launches"]),
                "clocks": h["clocks"], "parity": parity, "extra": extra}
        print(json.dumps(line), flush=True)
    for r_ in res.values():
        r_["batch"].close()
    for r in inst:
        r["idx"].close()
    if dist:
        dist.destroy_process_group()
    if parity_failed(parity):
        sys.exit("parity: GPU answers differ from the oracle's")


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "c4":
        run_batch(a)
    else:
        run_engine(a)


if __name__ == "__main__":
    main()
