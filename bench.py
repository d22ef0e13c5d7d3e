"""Benchmark of the two-electron matrix-element path (R^k + 2e-H assembly).

Workload (the "plain FP64 GPU drop-in at medium size" configuration): helium-like
Z=2, B-spline order 7, N=200 on the exp-linear knot grid to r_max=200 a.u.,
10 Gauss-Legendre points per interval, multipoles k=0..10, l_max=5, total
L=0..3 (natural parity), singlet and triplet, full blocks.  One step is the
whole path on the GPU: Slater primitives, the R^k store, the one-body matrices
and count + fill of all 8 symmetry blocks.

value : R^k elements/s = P^2 (max_k+1) / step time, outputs written into
        device buffers (inputs resident).  P = ordered band pairs = 2,558.
e2e   : same metric through the C ABI with host output buffers (pinned): the
        configuration lists go host->device and every CSR block device->host.
roofline: the CSR fill kernel (k_csr_fill), timed with CUDA events on the
        library's stream; algorithmic bytes = 24 B per stored H/S entry
        (int64 index + complex128 value) + the R^k tiles it stages.  traffic:
        DRAM bytes per launch, from the ncu capture of block 0 (profiles/
        k_csr_fill_order7_n200_block0.md) scaled to the average launch by
        algorithmic bytes.
cpu_baseline: the CPU oracle (C restatement of the reference, OpenMP) on a
        bounded sample: full Slater primitives + R^k map, and a row sample of
        every block extrapolated to the full block (one thread per block, the
        reference's OpenMP-over-symmetries decomposition).

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                [--precision fp64|mixed] [--no-e2e] [--no-cpu-baseline]
python bench.py --profile-block B   one radial pass and one count + fill of block B
                                    (0 = L=0 singlet, 117,620 rows): the small case
                                    for ncu captures of the fill kernel
python bench.py --workload batch    the ragged batch of 64 radial problems
                                    (tests/golden/ragged_problems.json): batched,
                                    graph-captured radial stage vs the same 64
                                    problems one handle after another
python bench.py --workload matvec   CSR mat-vec over the singlet H blocks of the
                                    default workload, assembled into HBM
python bench.py --workload order9_n800
                                    order 9, N=800, r_max=800, q=12, k=0..20,
                                    l_max=10, singlet L=0..5: radial stage, block
                                    counts and row samples of every block
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
METRIC = "R^k elements/s + 2e-H assembly s, mixed vs FP64 on GB300 at ≤1e-9 rel err"
WORKLOAD = dict(k=7, n_b=200, r_max=200.0, q=10, max_k=10, l_max=5, max_L=3, Z=2, spins=(0, 1),
                full=True, cap_order=2, cap_r0=10.0, cap_eta=1e-3)


# dram__bytes_read.sum + dram__bytes_write.sum of the k_csr_fill launch on
# block 0 (ncu --set full, profiles/k_csr_fill_order7_n200_block0.md) and that
# launch's algorithmic bytes (3,154,438,224 B of CSR + 20,100 staged tiles).
NCU_BLOCK0_DRAM = {"fp64": 3478840576.0, "mixed": 3683740672.0}
NCU_BLOCK0_ALG = 3453526224.0


def _pkg():
    sys.path.insert(0, ROOT)
    import __graft_entry__ as ge
    pkg = ge._package()
    if not os.path.exists(pkg.LIB_PATH):
        sys.path.insert(0, ge.PKG_DIR)
        import build as b
        b.build()
    return pkg


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def band_pairs(k, n_b):
    return n_b * (2 * k - 1) - k * (k - 1)


def workload_blocks(pkg, w):
    out = []
    for spin in w["spins"]:
        for (L, M, par) in pkg.basis.symmetries(w["max_L"], True):
            cf = pkg.configs(L, par, w["l_max"], w["n_b"], w["k"], spin=spin)
            out.append((L, par, spin, cf))
    return out


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------
# CPU baseline (oracle) on a bounded sample
# --------------------------------------------------------------------------
def cpu_baseline(pkg, w, rows_per_block=96, threads=None):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from concurrent.futures import ThreadPoolExecutor
    threads = threads or os.cpu_count()
    t = pkg.grids.explin_knots(w["k"], w["n_b"], w["r_max"])
    t0 = time.perf_counter()
    prim = O.slater(t, w["k"], w["q"], w["max_k"], nthreads=threads)
    t1 = time.perf_counter()
    R = O.rk_map(w["n_b"], w["k"], w["max_k"], prim)
    t2 = time.perf_counter()
    H1p = O.setup_H1p(t, w["k"], w["q"], w["Z"], w["l_max"] + 1, w["cap_order"], w["cap_r0"],
                      w["cap_eta"])
    S = O.setup_S(t, w["k"], w["q"])
    blocks = [(L, par, spin, O.count_configs(L, par, w["l_max"], w["n_b"], w["k"], spin=spin))
              for spin in w["spins"] for (L, M, par) in pkg.basis.symmetries(w["max_L"], True)]

    def run(b):
        L, par, spin, cf = b
        n = cf.size
        starts = np.linspace(0, n - 1, rows_per_block).astype(np.int64)
        ts = time.perf_counter()
        for r in starts:
            O.construct_block(cf, L, w["k"], w["n_b"], w["max_k"], R, H1p, S, w["full"], spin,
                              rows=(int(r), int(r) + 1))
        return (time.perf_counter() - ts) * n / rows_per_block

    t3 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=min(threads, len(blocks))) as ex:
        est = list(ex.map(run, blocks))
    t4 = time.perf_counter()
    t_full = (t1 - t0) + (t2 - t1) + max(est)
    P = band_pairs(w["k"], w["n_b"])
    elems = P * P * (w["max_k"] + 1)
    return dict(value=elems / t_full, unit="R^k elements/s", cores=threads, kind="port",
                sample=("full Slater primitives (%.1f s, OpenMP over k) + full R^k map (%.1f s, "
                        "serial) measured; assembly extrapolated from %d evenly spaced rows of each "
                        "of the %d blocks (%.1f s of sampling, one thread per block): full path "
                        "%.0f s" % (t1 - t0, t2 - t1, rows_per_block, len(blocks), t4 - t3, t_full)),
                t_full_s=t_full, t_slater_s=t1 - t0, t_rk_s=t2 - t1, t_assembly_s=max(est))


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def run_ours(args, rank, world):
    import torch
    pkg = _pkg()
    w = WORKLOAD
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    prec = pkg.PREC_MIXED if args.precision == "mixed" else pkg.PREC_FP64
    t = pkg.grids.explin_knots(w["k"], w["n_b"], w["r_max"])
    blocks = workload_blocks(pkg, w)
    h = pkg.Bs2e(t, w["k"], w["q"], w["max_k"], precision=prec, device=dev.index)
    stream = torch.cuda.ExternalStream(h.stream, device=dev)

    def radial():
        h.slater()
        h.rk()
        h.one_body(w["Z"], w["l_max"] + 1, w["cap_order"], w["cap_r0"], w["cap_eta"],
                   copy_out=False)

    radial()
    counts = [h.block_count(cf, L, w["full"], spin) for (L, par, spin, cf) in blocks]
    nH = sum(c[0] for c in counts)
    nS = sum(c[1] for c in counts)
    # device-resident outputs for every block
    out_dev = []
    for (L, par, spin, cf), (ch, cs) in zip(blocks, counts):
        n = cf.size
        Hd = dict(index_ptr=torch.empty(n + 1, dtype=torch.int64, device=dev),
                  indices=torch.empty(ch, dtype=torch.int64, device=dev),
                  data=torch.empty(ch, dtype=torch.complex128, device=dev))
        Sd = dict(index_ptr=torch.empty(n + 1, dtype=torch.int64, device=dev),
                  indices=torch.empty(cs, dtype=torch.int64, device=dev),
                  data=torch.empty(cs, dtype=torch.complex128, device=dev))
        out_dev.append((Hd, Sd))
    ptrs = [({x: v.data_ptr() for x, v in Hd.items()}, {x: v.data_ptr() for x, v in Sd.items()})
            for (Hd, Sd) in out_dev]
    tile_bytes = 8 * ((w["max_k"] + 1) * (2 * w["k"] - 1) ** 2 + 1) // 2 * 2
    n_tiles = sum(np.unique(cf["n1"] * 100000 + cf["n2"]).size for (_, _, _, cf) in blocks)
    fill_bytes = 24 * (nH + nS) + n_tiles * tile_bytes

    fill_ms = []

    def step_device(record):
        radial()
        for b, ((L, par, spin, cf), (Hp, Sp)) in enumerate(zip(blocks, ptrs)):
            h.block_count(cf, L, w["full"], spin)
            if record:
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            h.block_fill_into(cf, L, w["full"], spin, Hp, Sp, on_device=True)
            if record:
                e1.record(stream)
                fill_ms.append((e0, e1))

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(args.warmup):
        step_device(False)
    barrier()
    launches0 = h.launch_count
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with Clocks(dev.index) as clk:
        barrier()
        ev0.record(stream)
        for _ in range(args.steps):
            step_device(True)
        ev1.record(stream)
        barrier()
    launches = h.launch_count - launches0
    t_dev = ev0.elapsed_time(ev1) / 1e3
    fill_s = sum(a.elapsed_time(b) for a, b in fill_ms) / 1e3
    nb = len(blocks)
    per_block_ms = [sum(fill_ms[i][0].elapsed_time(fill_ms[i][1])
                        for i in range(j, len(fill_ms), nb)) / args.steps for j in range(nb)]
    t_dev = _max_over_ranks(t_dev, world)
    P = band_pairs(w["k"], w["n_b"])
    elems = P * P * (w["max_k"] + 1)
    value = world * elems * args.steps / t_dev
    # radial stage alone (slater + R^k + one-body), for the "+ 2e-H assembly s" split
    barrier()
    r0 = torch.cuda.Event(enable_timing=True)
    r1 = torch.cuda.Event(enable_timing=True)
    r0.record(stream)
    for _ in range(args.steps):
        radial()
    r1.record(stream)
    barrier()
    t_radial = r0.elapsed_time(r1) / 1e3 / args.steps

    if args.no_e2e:
        return _result(args, pkg, prec, world, blocks, nH, nS, elems, t_dev, t_radial, None,
                       launches, fill_bytes, fill_s, clk, h, rank, per_block_ms)
    # e2e through the C ABI with pinned host buffers
    del out_dev
    torch.cuda.empty_cache()
    host = []
    for (L, par, spin, cf), (ch, cs) in zip(blocks, counts):
        n = cf.size
        mk = lambda m, dt: torch.empty(m, dtype=dt, pin_memory=True).numpy()
        H = dict(index_ptr=mk(n + 1, torch.int64), indices=mk(ch, torch.int64),
                 data=mk(ch, torch.complex128))
        S = dict(index_ptr=mk(n + 1, torch.int64), indices=mk(cs, torch.int64),
                 data=mk(cs, torch.complex128))
        host.append((H, S))
    pinned_cfg = [torch.from_numpy(cf.view(np.int64).copy()).pin_memory().numpy().view(
        pkg.CONFIG_DTYPE) for (_, _, _, cf) in blocks]
    h2d = t.nbytes + sum(c.nbytes for c in pinned_cfg)
    d2h = sum(H["index_ptr"].nbytes + H["indices"].nbytes + H["data"].nbytes +
              S["index_ptr"].nbytes + S["indices"].nbytes + S["data"].nbytes for H, S in host)

    def step_e2e():
        radial()
        for (L, par, spin, _), cf, (H, S) in zip(blocks, pinned_cfg, host):
            h.block_count(cf, L, w["full"], spin)
            h.block_fill_into(cf, L, w["full"], spin, H, S, on_device=False)

    e2e_steps = max(1, min(args.steps, 3))
    step_e2e()
    barrier()
    te0 = time.perf_counter()
    for _ in range(e2e_steps):
        step_e2e()
    barrier()
    t_e2e = _max_over_ranks((time.perf_counter() - te0) / e2e_steps, world)
    # this box's device-to-host copy rate into the same pinned buffers: one
    # 4 GiB copy into the largest, and copies covering every byte of all of
    # them (the ceiling of the e2e number, which depends on the host pages)
    big = max((x for H, S in host for x in (H["data"], S["data"])), key=lambda a: a.nbytes)
    nbytes = min(big.nbytes, 4 << 30) // 16 * 16
    src = torch.empty(nbytes // 8, dtype=torch.float64, device=dev)
    dst = torch.from_numpy(big.view(np.float64)[:nbytes // 8])
    dst.copy_(src, non_blocking=True)
    torch.cuda.synchronize()
    tc0 = time.perf_counter()
    for _ in range(3):
        dst.copy_(src, non_blocking=True)
    torch.cuda.synchronize()
    d2h_gbs = 3 * nbytes / (time.perf_counter() - tc0) / 1e9
    srcb = src.view(torch.uint8)
    tc0 = time.perf_counter()
    tot_b = 0
    for H, S in host:
        for a in (H["index_ptr"], H["indices"], H["data"], S["index_ptr"], S["indices"], S["data"]):
            flat = torch.from_numpy(a.view(np.uint8).reshape(-1))
            for o in range(0, flat.numel(), nbytes):
                m = min(nbytes, flat.numel() - o)
                flat[o:o + m].copy_(srcb[:m], non_blocking=True)
                tot_b += m
    torch.cuda.synchronize()
    d2h_all_gbs = tot_b / (time.perf_counter() - tc0) / 1e9
    del src, srcb
    e2e = {"value": world * elems / t_e2e, "unit": "R^k elements/s",
           "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "s_per_step": t_e2e,
           "d2h_copy_gbs_this_box": d2h_gbs, "d2h_copy_gbs_all_buffers": d2h_all_gbs,
           "d2h_achieved_gbs": d2h / t_e2e / 1e9}
    return _result(args, pkg, prec, world, blocks, nH, nS, elems, t_dev, t_radial, e2e, launches,
                   fill_bytes, fill_s, clk, h, rank, per_block_ms)


def _result(args, pkg, prec, world, blocks, nH, nS, elems, t_dev, t_radial, e2e, launches,
            fill_bytes, fill_s, clk, h, rank, per_block_ms):
    w = WORKLOAD
    value = world * elems * args.steps / t_dev
    peak, peak_src = _peaks()
    achieved = fill_bytes * args.steps / fill_s / 1e9 if fill_s > 0 else None
    # DRAM bytes of an average fill launch: block 0's measured traffic per
    # algorithmic byte times the average launch's algorithmic bytes
    traffic = NCU_BLOCK0_DRAM[args.precision] / NCU_BLOCK0_ALG * fill_bytes / len(blocks)
    res = {
        "metric": METRIC, "value": value, "unit": "R^k elements/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == pkg.PREC_FP64 else "f64 out, f32-pair k-sum",
        "data": "synthetic (deterministic knot grid, no dataset)",
        "config": {"workload": "k=7 N=200 r_max=200 q=10 k=0..10 l_max=5 L=0..3 "
                               "singlet+triplet full blocks (8 blocks, %d rows)" %
                               sum(cf.size for (_, _, _, cf) in blocks),
                   "precision": args.precision, "nnz_H": nH, "nnz_S": nS,
                   "rk_elements_per_step": elems,
                   "l2": "every step writes %.1f GB of CSR (> L2)" % (24 * (nH + nS) / 1e9)},
        "assembly_s": (t_dev / args.steps) - t_radial,
        "radial_s": t_radial,
        "rk_stage_elements_per_s": elems / t_radial,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "k_csr_fill", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                     "traffic": traffic, "peak_source": peak_src,
                     "algorithmic_bytes_per_launch": fill_bytes / len(blocks),
                     "launches_per_step": len(blocks),
                     "fill_s_per_step": fill_s / args.steps,
                     "fill_ms_per_block": per_block_ms},
        "clocks": clk.summary(),
    }
    h.close()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        res["cpu_baseline"] = {k: v for k, v in cpu_baseline(pkg, w).items()
                               if k in ("value", "unit", "cores", "kind", "sample")}
    return res


def profile_block(args):
    """Small case for ncu: one radial pass, then count + fill of one block into
    device buffers (block 0 writes ~2.9 GB of CSR, above L2, one k_fill launch)."""
    import torch
    pkg = _pkg()
    w = WORKLOAD
    prec = pkg.PREC_MIXED if args.precision == "mixed" else pkg.PREC_FP64
    t = pkg.grids.explin_knots(w["k"], w["n_b"], w["r_max"])
    L, par, spin, cf = workload_blocks(pkg, w)[args.profile_block]
    with pkg.Bs2e(t, w["k"], w["q"], w["max_k"], precision=prec) as h:
        h.slater()
        h.rk()
        h.one_body(w["Z"], w["l_max"] + 1, w["cap_order"], w["cap_r0"], w["cap_eta"],
                   copy_out=False)
        ch, cs = h.block_count(cf, L, w["full"], spin)
        n = cf.size
        dev = torch.device("cuda", 0)
        Hd = dict(index_ptr=torch.empty(n + 1, dtype=torch.int64, device=dev),
                  indices=torch.empty(ch, dtype=torch.int64, device=dev),
                  data=torch.empty(ch, dtype=torch.complex128, device=dev))
        Sd = dict(index_ptr=torch.empty(n + 1, dtype=torch.int64, device=dev),
                  indices=torch.empty(cs, dtype=torch.int64, device=dev),
                  data=torch.empty(cs, dtype=torch.complex128, device=dev))
        torch.cuda.synchronize()
        h.block_fill_into(cf, L, w["full"], spin, {x: v.data_ptr() for x, v in Hd.items()},
                          {x: v.data_ptr() for x, v in Sd.items()}, on_device=True)
        h.synchronize()
        print(json.dumps({"profile_block": args.profile_block, "L": L, "spin": spin,
                          "rows": int(n), "nnz_H": ch, "nnz_S": cs,
                          "output_bytes": 24 * (ch + cs)}))


def run_batch(args):
    """The ragged batch of 64 radial problems: the batched, graph-captured
    radial stage (bs2e_batch_run) against the same handles run one after
    another through bs2e_slater + bs2e_rk; both produce bit-identical stores."""
    import torch
    pkg = _pkg()
    probs = json.load(open(os.path.join(ROOT, "tests", "golden", "ragged_problems.json")))
    prec = pkg.PREC_MIXED if args.precision == "mixed" else pkg.PREC_FP64
    hs = [pkg.Bs2e(pkg.grids.explin_knots(p["k"], p["n_b"], p["r_max"]), p["k"], p["k_GL"],
                   p["max_k"], precision=prec) for p in probs]
    elems = sum(band_pairs(p["k"], p["n_b"]) ** 2 * (p["max_k"] + 1) for p in probs)
    store_bytes = sum(p["n_b"] ** 2 * (((p["max_k"] + 1) * (2 * p["k"] - 1) ** 2 + 1) // 2 * 2) * 8
                      for p in probs)

    def fingerprint(sel):
        out = []
        for i in sel:
            h = hs[i]
            W = 2 * h.k - 1
            buf = torch.empty(h.n_b * h.n_b * W * W, dtype=torch.float64, device="cuda")
            acc = 0
            for kk in range(h.K1):
                h.rk_export(kk, buf.data_ptr(), on_device=True)
                acc ^= int(buf.view(torch.int64).sum().item()) & ((1 << 63) - 1)
            out.append(acc)
        return out

    sel = [0, len(hs) // 2, len(hs) - 1]
    batch = pkg.RadialBatch(hs)
    t0 = time.perf_counter()
    batch.run()  # tuning + graph capture
    t_first = time.perf_counter() - t0
    for _ in range(max(0, args.warmup - 1)):
        batch.run()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        batch.run()
    t_batch = (time.perf_counter() - t0) / args.steps
    fp_batch = fingerprint(sel)
    for _ in range(args.warmup):
        for h in hs:
            h.slater()
            h.rk()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for h in hs:
            h.slater()
            h.rk()
    t_seq = (time.perf_counter() - t0) / args.steps
    fp_seq = fingerprint(sel)
    tun = batch.tuning()
    batch.close()
    for h in hs:
        h.close()
    return {
        "metric": "R^k elements/s, ragged batch of 64 radial problems", "impl": "ours",
        "value": elems / t_batch, "unit": "R^k elements/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_batch, "higher_is_better": True,
        "dtype": "f64" if prec == pkg.PREC_FP64 else "f64 sums, f32-pair store",
        "data": "synthetic: 64 problems from numpy default_rng(0), tests/golden/ragged_problems.json",
        "config": {"workload": "ragged batch: order in {6,7,8}, N in [100,500], r_max=N, "
                               "max_k in [4,16], k_GL=k+4", "rk_elements_per_step": elems,
                   "store_bytes": store_bytes, "timing": "wall clock, each run synchronised"},
        "sequential": {"value": elems / t_seq, "ms_per_step": 1e3 * t_seq,
                       "launches_per_step": 4 * len(hs)},
        "speedup_vs_sequential": t_seq / t_batch,
        "first_run_s": t_first, "tuning": tun,
        "bit_identical_sample": fp_batch == fp_seq,
    }


LARGE = dict(k=9, n_b=800, r_max=800.0, q=12, max_k=20, l_max=10, max_L=5, Z=2, cap_order=2,
               cap_r0=10.0, cap_eta=1e-3)


def run_large(args, sample_rows=2048):
    """The large configuration (order 9, N=800, r_max=800, 12 GL points,
    k=0..20, l_max=10, singlet L=0..5 with the L+-1 dipole blocks, q=0).  Its
    CSR (terabytes) exceeds HBM and host memory, so: the radial stage and the
    exact non-zero counts of every block are measured in full; H/S assembly
    and dipole blocks are timed on row samples (3 ranges per block) and the
    full-block time is extrapolated from the sample rate; the mixed path is
    compared with the FP64 path on the same samples."""
    import torch
    pkg = _pkg()
    w = LARGE
    dev = torch.device("cuda", 0)
    t = pkg.grids.explin_knots(w["k"], w["n_b"], w["r_max"])
    syms = pkg.basis.symmetries(w["max_L"], True)
    cfs = [(L, M, par, pkg.configs(L, par, w["l_max"], w["n_b"], w["k"])) for (L, M, par) in syms]
    out = {"metric": "large configuration: R^k stage, counts, sampled assembly", "config": {
        "workload": "k=9 N=800 r_max=800 q=12 k=0..20 l_max=10 singlet L=0..5 + dipole L+-1 (q=0)",
        "rows": [int(cf.size) for (_, _, _, cf) in cfs], "sample_rows_per_range": sample_rows},
        "data": "synthetic (deterministic knot grid, no dataset)"}
    P = band_pairs(w["k"], w["n_b"])
    elems = P * P * (w["max_k"] + 1)
    hs = {}
    for name, prec in (("fp64", pkg.PREC_FP64), ("mixed", pkg.PREC_MIXED)):
        h = pkg.Bs2e(t, w["k"], w["q"], w["max_k"], precision=prec)
        stream = torch.cuda.ExternalStream(h.stream, device=dev)

        def radial():
            h.slater()
            h.rk()
            h.one_body(w["Z"], w["l_max"] + 1, w["cap_order"], w["cap_r0"], w["cap_eta"],
                       copy_out=False)
        radial()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        radial()
        e1.record(stream)
        torch.cuda.synchronize()
        out["radial_s_" + name] = e0.elapsed_time(e1) / 1e3
        hs[name] = (h, stream)
    out["rk_elements"] = elems
    out["rk_elements_per_s_fp64"] = elems / out["radial_s_fp64"]
    out["rk_store_bytes"] = int(w["n_b"] ** 2 * (((w["max_k"] + 1) * (2 * w["k"] - 1) ** 2 + 1) // 2 * 2) * 8)
    blocks = []
    tot_s = {"fp64": 0.0, "mixed": 0.0}
    worst = 0.0
    worst_max = 0.0
    for (L, M, par, cf) in cfs:
        n = cf.size
        b = {"L": L, "rows": int(n)}
        t0 = time.perf_counter()
        nH, nS = hs["fp64"][0].block_count(cf, L, True, 0)
        b["count_s"] = time.perf_counter() - t0
        b["nnz_H"], b["nnz_S"] = int(nH), int(nS)
        b["csr_bytes"] = 24 * (nH + nS) + 16 * (n + 1)
        samples = {}
        for name in ("fp64", "mixed"):
            h, stream = hs[name]
            h.block_count(cf, L, True, 0)
            ent, ms = 0, 0.0
            vals = []
            for frac in (0.05, 0.5, 0.9):
                r0 = int(frac * n)
                cnt = min(sample_rows, n - r0)
                sh, ss = h.block_count_rows(cf, L, r0, cnt, True, 0)
                bufs = [torch.empty(cnt + 1, dtype=torch.int64, device=dev),
                        torch.empty(sh, dtype=torch.int64, device=dev),
                        torch.empty(sh, dtype=torch.complex128, device=dev),
                        torch.empty(cnt + 1, dtype=torch.int64, device=dev),
                        torch.empty(ss, dtype=torch.int64, device=dev),
                        torch.empty(ss, dtype=torch.complex128, device=dev)]
                Hd = dict(index_ptr=bufs[0].data_ptr(), indices=bufs[1].data_ptr(),
                          data=bufs[2].data_ptr())
                Sd = dict(index_ptr=bufs[3].data_ptr(), indices=bufs[4].data_ptr(),
                          data=bufs[5].data_ptr())
                h.block_rows_into(cf, L, r0, cnt, True, 0, Hd, Sd)  # warm
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize()
                e0.record(stream)
                h.block_rows_into(cf, L, r0, cnt, True, 0, Hd, Sd)
                e1.record(stream)
                torch.cuda.synchronize()
                ms += e0.elapsed_time(e1)
                ent += sh + ss
                vals.append((bufs[1].cpu(), bufs[2].cpu(), bufs[4].cpu(), bufs[5].cpu()))
                del bufs
            rate = ent / (ms / 1e3)
            samples[name] = vals
            b["sample_entries_per_s_" + name] = rate
            b["assembly_s_extrapolated_" + name] = (nH + nS) / rate
            tot_s[name] += (nH + nS) / rate
        same = True
        rel = 0.0  # |mixed - fp64| / |fp64| over entries >= 1e-10 of the sample's largest
        rel_max = 0.0  # |mixed - fp64| / largest |fp64| of the sample range
        for (i1, d1, si1, sd1), (i2, d2, si2, sd2) in zip(samples["fp64"], samples["mixed"]):
            same = same and torch.equal(i1, i2) and torch.equal(si1, si2)
            for x, y in ((d1, d2), (sd1, sd2)):
                ax = x.abs()
                if ax.numel() == 0:
                    continue
                top = float(ax.max())
                mask = ax >= 1e-10 * top
                if mask.any():
                    rel = max(rel, float(((y - x).abs()[mask] / ax[mask]).max()))
                if top > 0:
                    rel_max = max(rel_max, float((y - x).abs().max()) / top)
        b["pattern_identical_mixed_vs_fp64"] = bool(same)
        b["max_err_rel_to_entry_mixed_vs_fp64"] = rel
        b["max_err_rel_to_sample_max_mixed_vs_fp64"] = rel_max
        worst = max(worst, rel)
        worst_max = max(worst_max, rel_max)
        blocks.append(b)
        torch.cuda.empty_cache()
    out["blocks"] = blocks
    out["assembly_s_extrapolated_fp64"] = tot_s["fp64"]
    out["assembly_s_extrapolated_mixed"] = tot_s["mixed"]
    # Relative to the entry, a value that cancels between the multipole terms
    # shows the terms' rounding magnified; the 1e-9 bar is relative to the
    # term magnitude, which tests/test_precision_report.py checks against the
    # oracle on these blocks.
    out["max_err_rel_to_entry_mixed_vs_fp64"] = worst
    out["max_err_rel_to_sample_max_mixed_vs_fp64"] = worst_max
    # dipole blocks L -> L+1, q = 0 (z polarisation), length gauge
    h = hs["fp64"][0]
    h.radial_dipole(0, copy_out=False)
    dips = []
    for (L1, M1, p1, cf1), (L2, M2, p2, cf2) in zip(cfs[:-1], cfs[1:]):
        t0 = time.perf_counter()
        nd = h.dip_block_count(cf1, (L1, M1, p1), cf2, (L2, M2, p2), 0)
        tc = time.perf_counter() - t0
        r0 = cf1.size // 2
        rows = cf1[r0:r0 + sample_rows]
        h.dip_block(rows, (L1, M1, p1), cf2, (L2, M2, p2), 0)  # warm
        t0 = time.perf_counter()
        D = h.dip_block(rows, (L1, M1, p1), cf2, (L2, M2, p2), 0)
        ts = time.perf_counter() - t0
        rate = D["nnz"] / ts if ts > 0 else None
        dips.append({"L": [L1, L2], "nnz": int(nd), "count_s": tc, "sample_nnz": int(D["nnz"]),
                     "sample_s_host_outputs": ts,
                     "fill_s_extrapolated": (nd / rate) if rate else None})
    out["dipole_blocks"] = dips
    for (h, _) in hs.values():
        h.close()
    return out


def run_matvec(args):
    """CSR_mv / CSR_mv_sym (bs2e_csr_mv on device pointers) over the H blocks of
    the bench workload, assembled into HBM by the library: achieved GB/s of
    the mat-vec kernel against the measured copy bandwidth."""
    import torch
    pkg = _pkg()
    w = WORKLOAD
    dev = torch.device("cuda", 0)
    prec = pkg.PREC_MIXED if args.precision == "mixed" else pkg.PREC_FP64
    t = pkg.grids.explin_knots(w["k"], w["n_b"], w["r_max"])
    blocks = workload_blocks(pkg, w)
    res = {}
    with pkg.Bs2e(t, w["k"], w["q"], w["max_k"], precision=prec) as h:
        h.slater()
        h.rk()
        h.one_body(w["Z"], w["l_max"] + 1, w["cap_order"], w["cap_r0"], w["cap_eta"],
                   copy_out=False)
        stream = torch.cuda.ExternalStream(h.stream, device=dev)
        for op, full, name in ((0, True, "csr_mv"), (2, False, "csr_mv_sym")):
            t_ms, nbytes, nnz_all, cplx_all = 0.0, 0, 0, 0.0
            for (L, par, spin, cf) in blocks[:4]:
                nH, nS = h.block_count(cf, L, full, spin)
                n = cf.size
                ptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
                idx = torch.empty(nH, dtype=torch.int64, device=dev)
                dat = torch.empty(nH, dtype=torch.complex128, device=dev)
                sp = torch.empty(n + 1, dtype=torch.int64, device=dev)
                si = torch.empty(nS, dtype=torch.int64, device=dev)
                sd = torch.empty(nS, dtype=torch.complex128, device=dev)
                h.block_fill_into(cf, L, full, spin,
                                  dict(index_ptr=ptr.data_ptr(), indices=idx.data_ptr(),
                                       data=dat.data_ptr()),
                                  dict(index_ptr=sp.data_ptr(), indices=si.data_ptr(),
                                       data=sd.data_ptr()), on_device=True)
                del si, sd, sp
                cplx = float((dat.imag != 0).double().mean().item())
                x = torch.randn(n, dtype=torch.complex128, device=dev)
                y = torch.empty(n, dtype=torch.complex128, device=dev)
                args_ = (op, n, n, nH, ptr.data_ptr(), idx.data_ptr(), dat.data_ptr(),
                         x.data_ptr(), y.data_ptr())
                torch.cuda.synchronize()  # x is made on torch's stream, read on the library's
                for _ in range(args.warmup):
                    h.csr_mv_device(*args_)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize()
                e0.record(stream)
                for _ in range(args.steps):
                    h.csr_mv_device(*args_)
                e1.record(stream)
                torch.cuda.synchronize()
                t_ms += e0.elapsed_time(e1) / args.steps
                # algorithmic bytes: int64 column + complex128 value per entry,
                # two row pointers per row, x read once and y written once
                nbytes += 24 * nH + 8 * (n + 1) + 32 * n
                nnz_all += nH
                cplx_all = cplx_all + cplx * nH
                del ptr, idx, dat, x, y
                torch.cuda.empty_cache()
            peak, src = _peaks()
            gbs = nbytes / (t_ms / 1e3) / 1e9
            res[name] = {"ms_per_product_all_blocks": t_ms, "nnz": nnz_all, "bytes": nbytes,
                         "fraction_complex_entries": cplx_all / max(nnz_all, 1),
                         "achieved_gbs": gbs, "frac_of_measured_hbm": gbs / peak,
                         "peak_source": src}
    return {"metric": "H x: CSR mat-vec over the L=0..3 singlet H blocks", "results": res,
            "config": {"workload": "k=7 N=200 r_max=200 q=10 k=0..10 l_max=5 L=0..3 singlet",
                       "precision_of_blocks": args.precision},
            "steps": args.steps, "warmup": args.warmup}


def _max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    """The reference's algorithm on the host cores (the oracle port), same metric."""
    pkg = _pkg()
    w = WORKLOAD
    for _ in range(args.warmup):
        cpu_baseline(pkg, w, rows_per_block=8)
    vals = []
    last = None
    for _ in range(args.steps):
        last = cpu_baseline(pkg, w)
        vals.append(last["value"])
    v = statistics.median(vals)
    return {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "R^k elements/s",
        "n_gpus": args.gpus, "gpus_used": 0,  # the run's N; the arm itself runs on host cores
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * last["t_full_s"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (deterministic knot grid, no dataset)",
        "config": {"workload": "k=7 N=200 r_max=200 q=10 k=0..10 l_max=5 L=0..3 "
                               "singlet+triplet full blocks (8 blocks)"},
        "cpu_baseline": {"value": v, "unit": "R^k elements/s", "cores": last["cores"],
                         "kind": "port", "sample": last["sample"]},
        "e2e": {"value": v, "unit": "R^k elements/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--profile-block", type=int, default=None)
    ap.add_argument("--workload", default="order7_n200",
                    choices=["order7_n200", "batch", "matvec", "order9_n800"])
    args = ap.parse_args()
    if args.profile_block is not None:
        profile_block(args)
        return
    if args.workload == "batch":
        print(json.dumps(run_batch(args)), flush=True)
        return
    if args.workload == "matvec":
        print(json.dumps(run_matvec(args)), flush=True)
        return
    if args.workload == "order9_n800":
        print(json.dumps(run_large(args)), flush=True)
        return
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    res = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
