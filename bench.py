"""Benchmark of the two-electron matrix-element path (R^k + 2e-H assembly).

Default workload, the large form: helium-like Z=2, B-spline order 9, N=800 on
the exp-linear knot grid to r_max=800 a.u., 12 Gauss-Legendre points per
interval, multipoles k=0..20, l_max=10, singlet L=0..5 (natural parity), full
blocks, with the L -> L+1 dipole blocks (q=0, length gauge).  One job is the
whole path on the GPU: Slater primitives, the R^k store (3.84e9 elements,
31 GB), one-body and radial dipole matrices, the count pass of every block,
and the assembly of the 6 symmetry blocks (5.3e11 H and S entries) and the
5 dipole blocks (~6e10 entries): ~14 TB of CSR, more than HBM and host memory
together.  The CSR is therefore made in n1 bands (bs2e_block_fill_band) and
dipole row slices of at most one staging area (24 GiB; two areas in turn)
and consumed on the device as it is made, on a second stream while the next
band fills: the mat-vec bs2e_csr_mv applies every band of H and S and every
slice of D to a fixed vector (the product a solver needs), or with
--consume digest a 64-bit wrapping sum of every word of every band and slice
(pointers, columns and the bit patterns of the values) reads them instead.
Either way a chunk made again must give the same sum.

A bench step is 1/16 of a job: the job's bands and slices cut into 16
chunks of nearly equal CSR bytes, chunk 0 also running the radial stage, so
K steps process K/16 jobs and the timed region of K >= 16 steps holds at
least one whole job, whose time is reported as job_s.

value : R^k elements per job x jobs done / time (device-resident inputs and
        outputs; jobs done counted by CSR bytes of the chunks run).
e2e   : the same chunks through the C ABI with HOST buffers: configuration
        lists from pinned host memory, every band and slice copied into
        pinned host buffers (bs2e_block_fill_band / bs2e_dip_block_fill with
        host outputs), a chunk's units alternating between two handles of
        the same basis (one thread each) so that one band's copy to the host
        runs beside the next band's fill.
mixed : the same job on the mixed-precision path (BS2E_PREC_MIXED), its time,
        and the errors of both paths against the oracle (and of mixed against
        FP64) on rows sampled across the blocks.
roofline: the band fill (k_csr_fill), timed with CUDA events on the
        library's stream; algorithmic bytes = 24 B per stored H/S entry + the
        band's 1-based pointers + the R^k tiles it stages; traffic = DRAM
        bytes per algorithmic byte of an ncu capture of one band, scaled.
cpu_baseline / --impl reference: the CPU oracle (the C restatement of the
        reference, all host threads) on the same fraction f of every stage of
        the job -- f of the R^k tiles, of every block's rows and of every
        dipole block's rows -- so value = f x R^k elements / time.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                [--precision fp64|mixed] [--workload order9_n800|order7_n200|...]
python bench.py --workload order7_n200   the medium drop-in size (order 7, N=200,
                                         k=0..10, l_max=5, L=0..3, singlet and
                                         triplet), whole blocks into HBM
python bench.py --profile-band B         one band fill of the large form (small
                                         case for ncu captures of k_csr_fill)
python bench.py --profile-dip B          one dipole row slice (block B -> B+1) of the
                                         large form's method (small case for k_dip_fill)
python bench.py --profile-block B        one whole-block fill of the medium size
                [--profile-mv]           (and one CSR_mv of its H: small case for ncu)
python bench.py --workload batch         the ragged batch of 64 radial problems
python bench.py --workload matvec        CSR mat-vec over medium-size H blocks
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
METRIC = "R^k elements/s + 2e-H assembly s, mixed vs FP64 on GB300 at ≤1e-9 rel err"

LARGE = dict(name="order9_n800", k=9, n_b=800, r_max=800.0, q=12, max_k=20, l_max=10,
             max_L=5, Z=2, spins=(0,), dipoles=True, cap_order=2, cap_r0=10.0, cap_eta=1e-3,
             area_bytes=24 << 30, n_chunks=16, cpu_frac=3 / 640000)
MEDIUM = dict(name="order7_n200", k=7, n_b=200, r_max=200.0, q=10, max_k=10, l_max=5,
              max_L=3, Z=2, spins=(0, 1), dipoles=False, cap_order=2, cap_r0=10.0,
              cap_eta=1e-3, n_chunks=1, cpu_frac=1e-2)
WORKLOADS = {"order9_n800": LARGE, "order7_n200": MEDIUM}

# DRAM bytes per algorithmic byte of the band fill, from one ncu capture of
# one band of the large form per precision (the figures and the command are
# in the profile summaries kept with this repository); None until captured.
FILL_TRAFFIC_RATIO = {"order9_n800": {"fp64": (23052800.0 + 2262179000.0) / 2342289120.0,
                                      "mixed": (25177600.0 + 2264250000.0) / 2342289120.0},
                      "order7_n200": {"fp64": 3478840576.0 / 3453526224.0,
                                      "mixed": 3683740672.0 / 3453526224.0}}


def workload_string(w):
    """The workload as both arms print it."""
    if w["name"] == "order9_n800":
        return ("order 9, N=800, r_max=800, q=12, k=0..20, l_max=10, singlet L=0..5 full "
                "blocks + dipole blocks L->L+1 (q=0, length gauge)")
    return ("order 7, N=200, r_max=200, q=10, k=0..10, l_max=5, L=0..3 singlet+triplet full "
            "blocks")


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


def rk_elements(w):
    return band_pairs(w["k"], w["n_b"]) ** 2 * (w["max_k"] + 1)


def tile_doubles(w):
    return ((w["max_k"] + 1) * (2 * w["k"] - 1) ** 2 + 1) // 2 * 2


def block_list(pkg, w):
    """[(L, M, parity, spin, configs)] in init_basis order, singlet then triplet."""
    out = []
    for spin in w["spins"]:
        for (L, M, par) in pkg.basis.symmetries(w["max_L"], True):
            out.append((L, M, par, spin, pkg.configs(L, par, w["l_max"], w["n_b"], w["k"],
                                                     spin=spin)))
    return out


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []

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
# CPU: the oracle on the same fraction f of every stage
# --------------------------------------------------------------------------
class CpuSample:
    """The reference's algorithm (the oracle) on a fraction f of the job's work
    units: f of the N^2 R^k tiles (rk_tiles: the tile's primitives and the
    reference's summation of them), f of the rows of every symmetry block
    (construct_block: the reference's O(n_config) loop per row) and f of the
    rows of every dipole block (construct_dip_block_tensor per row).  The
    one-body and radial dipole matrices (O(N k q) work) and the R^k tiles the
    sampled rows read (the R^k stage's other units) are prepared untimed.
    Every stage gets the same fraction, so the sample is f of the job."""

    def __init__(self, pkg, w, threads=None):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        self.O = O
        self.pkg = pkg
        self.w = w
        self.threads = threads or os.cpu_count() or 1
        self.t = pkg.grids.explin_knots(w["k"], w["n_b"], w["r_max"])
        self.blocks = block_list(pkg, w)
        self.H1p = O.setup_H1p(self.t, w["k"], w["q"], w["Z"], w["l_max"] + 1, w["cap_order"],
                               w["cap_r0"], w["cap_eta"])
        self.S = O.setup_S(self.t, w["k"], w["q"])
        self.mats = O.setup_radial_dip(self.t, w["k"], w["q"], 0) if w["dipoles"] else None

    def _rows(self, n, f, rng):
        m = max(1, int(round(f * n)))
        return np.sort(rng.choice(n, size=m, replace=False)), m / n

    def run(self, f, seed):
        from concurrent.futures import ThreadPoolExecutor
        O, w = self.O, self.w
        N, k = w["n_b"], w["k"]
        key = (f, seed)
        if getattr(self, "_key", None) != key:
            self._prep = self._prepare(f, seed)
            self._key = key
        tiles, jobs, dip_jobs, fracs, T, tab = self._prep
        n_t = len(tiles)
        # timed: f of each stage
        t0 = time.perf_counter()
        O.rk_tiles(self.t, k, w["q"], w["max_k"], tiles, nthreads=self.threads)
        t1 = time.perf_counter()

        def row(j):
            cf, L, spin, r = j
            O.construct_block(cf, L, k, N, w["max_k"], T, self.H1p, self.S, True, spin,
                              rows=(r, r + 1), tile_of=tab)

        def drow(j):
            (L1, M1, p1, _, c1), (L2, M2, p2, _, c2), r = j
            O.dip_block(c1[r:r + 1], (L1, M1, p1), c2, (L2, M2, p2), 0, True, k, N, 0, self.S,
                        self.mats)

        with ThreadPoolExecutor(max_workers=self.threads) as ex:
            list(ex.map(row, jobs))
            t2 = time.perf_counter()
            list(ex.map(drow, dip_jobs))
        t3 = time.perf_counter()
        t_all = t3 - t0
        elems = rk_elements(w)
        return {"value": f * elems / t_all, "unit": "R^k elements/s", "cores": self.threads,
                "kind": "port", "f": f, "t_s": t_all,
                "sample": ("fraction f=%.3g of every stage of one job on %d host threads: %d of "
                           "%d R^k tiles (%.2f s), %d block rows (%.2f s), %d dipole rows "
                           "(%.2f s); per-stage fractions %.3g..%.3g; full job %.0f s at this "
                           "rate (not measured)" %
                           (f, self.threads, n_t, N * N, t1 - t0, len(jobs), t2 - t1,
                            len(dip_jobs), t3 - t2, min(fracs + [n_t / N / N]),
                            max(fracs + [n_t / N / N]), t_all / f))}

    def _prepare(self, f, seed):
        """The sample's work units and, untimed, the R^k tiles its rows read."""
        O, w = self.O, self.w
        N, k = w["n_b"], w["k"]
        rng = np.random.default_rng(seed)
        n_t = max(1, int(round(f * N * N)))
        flat = rng.choice(N * N, size=n_t, replace=False)
        tiles = np.stack([flat // N + 1, flat % N + 1], axis=1)
        jobs, dip_jobs, fracs = [], [], []
        need = set()
        for (L, M, par, spin, cf) in self.blocks:
            rows, fb = self._rows(cf.size, f, rng)
            fracs.append(fb)
            for r in rows:
                need.add((int(cf["n1"][r]), int(cf["n2"][r])))
                jobs.append((cf, L, spin, int(r)))
        if w["dipoles"]:
            singlet = [b for b in self.blocks if b[3] == 0]
            for (b1, b2) in zip(singlet[:-1], singlet[1:]):
                rows, fb = self._rows(b1[4].size, f, rng)
                fracs.append(fb)
                for r in rows:
                    dip_jobs.append((b1, b2, int(r)))
        need = np.array(sorted(need), dtype=np.int64)
        T = O.rk_tiles(self.t, k, w["q"], w["max_k"], need, nthreads=self.threads)
        tab = O.tile_table(N, need)
        return tiles, jobs, dip_jobs, fracs, T, tab


# --------------------------------------------------------------------------
# GPU: the large form in bands and dipole slices
# --------------------------------------------------------------------------
class LargeJob:
    """The large form on one handle: planned bands and dipole slices, cut into
    chunks; run_chunk(j) assembles chunk j into the two staging areas and
    applies it to fixed vectors with the library's mat-vec."""

    def __init__(self, pkg, w, prec, areas, rank=0, world=1, plan=None, consume="mv"):
        import torch
        self.torch = torch
        self.pkg, self.w = pkg, w
        self.consume = consume
        self.digests = {}  # chunk -> [device sum of each run: int64 digest or complex y sum]
        self.dev = torch.device("cuda", torch.cuda.current_device())
        t = pkg.grids.explin_knots(w["k"], w["n_b"], w["r_max"])
        self.h = pkg.Bs2e(t, w["k"], w["q"], w["max_k"], precision=prec,
                          device=self.dev.index, stage_bytes=w["area_bytes"])
        self.h.set_block_cache(0)
        self.stream = torch.cuda.ExternalStream(self.h.stream, device=self.dev)
        # the consumer: a second handle (any basis; it only lends its stream
        # to the digest sums, or runs the mat-vec on device pointers) whose
        # stream works while the next band fills.  Both streams keep the
        # default priority.  Jobs timed back to back on one GB300 took
        # 8.74-8.87 s this way, 9.21-9.43 s with the consumer at the highest
        # priority, and 8.64 or 9.62 s with the fill's stream at the highest.
        self.hc = pkg.Bs2e(pkg.grids.explin_knots(6, 24, 20.0), 6, 8, 0, device=self.dev.index)
        self.cstream = torch.cuda.ExternalStream(self.hc.stream, device=self.dev)
        self.areas = areas
        self.blocks = [(L, M, par, spin, self._pin(cf)) for (L, M, par, spin, cf)
                       in block_list(pkg, w)]
        self.radial()
        self.plan = plan if plan is not None else self._plan(rank, world)
        units = [u for u in self.plan["units"] if u["owner"] == rank]
        seen = set()
        for u in units:  # the count pass of a block runs before its first band here
            u["count_first"] = u["kind"] == "band" and u["block"] not in seen
            if u["kind"] == "band":
                seen.add(u["block"])
        self.chunks = self._chunks(units, w["n_chunks"])
        g = torch.Generator(device="cpu").manual_seed(7)
        self.x = [torch.randn(cf.size, dtype=torch.complex128, generator=g).to(self.dev)
                  for (*_, cf) in self.blocks]
        maxr = max([u["rows"] for u in units] + [1])
        self.y = torch.empty(maxr, dtype=torch.complex128, device=self.dev)
        self.ysum = torch.zeros((), dtype=torch.complex128, device=self.dev)
        torch.cuda.synchronize()

    def _pin(self, cf):
        t = self.torch.from_numpy(cf.view(np.int64).reshape(-1).copy()).pin_memory()
        self._pinned = getattr(self, "_pinned", []) + [t]
        return t.numpy().view(self.pkg.CONFIG_DTYPE).reshape(-1)

    def radial(self, h=None):
        w, h = self.w, (self.h if h is None else h)
        h.slater()
        h.rk()
        h.one_body(w["Z"], w["l_max"] + 1, w["cap_order"], w["cap_r0"], w["cap_eta"],
                   copy_out=False)
        if w["dipoles"]:
            h.radial_dipole(0, copy_out=False)

    def _plan(self, rank, world):
        pkg, w, h = self.pkg, self.w, self.h
        N = w["n_b"]
        per, tiles = [], []
        for (L, M, par, spin, cf) in self.blocks:
            r, nh, ns, p = h.band_count(cf, L, 1, N, True, spin, per_n1=True)
            per.append(p)
            # staged tiles per n1: distinct (n1, n2) of the block's rows
            key = np.unique(cf["n1"].astype(np.int64) * (N + 1) + cf["n2"])
            tiles.append(np.bincount(key // (N + 1), minlength=N + 1)[1:])
        # room for 256-byte alignment of six arrays and a rows list per band
        bands = pkg.band_plan(per, w["area_bytes"] - (64 << 20), world)
        units = []
        for (b, a, m, owner, nbytes) in bands:
            p = per[b][a - 1:a - 1 + m]
            units.append(dict(kind="band", block=int(b), n1=int(a), m=int(m), owner=int(owner),
                              bytes=int(nbytes), rows=int(p[:, 0].sum()),
                              nH=int(p[:, 1].sum()), nS=int(p[:, 2].sum()),
                              tiles=int(tiles[b][a - 1:a - 1 + m].sum())))
        if w["dipoles"]:
            load = np.zeros(world)
            for u in units:
                load[u["owner"]] += u["bytes"]
            singlet = [i for i, b in enumerate(self.blocks) if b[3] == 0]
            dips = []
            for i1, i2 in zip(singlet[:-1], singlet[1:]):
                dips += self._dip_slices(i1, i2)
            for d in sorted(dips, key=lambda d: -d["bytes"]):
                d["owner"] = int(np.argmin(load))
                load[d["owner"]] += d["bytes"]
            units += dips
        return {"units": units}

    def _dip_slices(self, i1, i2):
        """Row slices of the dipole block (i1 -> i2) whose CSR fits the area."""
        h, w = self.h, self.w
        (L1, M1, p1, _, c1), (L2, M2, p2, _, c2) = self.blocks[i1], self.blocks[i2]
        cap = w["area_bytes"] - (1 << 20)
        out, todo = [], [(0, c1.size)]
        total = h.dip_block_count(c1, (L1, M1, p1), c2, (L2, M2, p2), 0)
        if total:
            step = max(1, int(c1.size * 0.8 * cap / (24 * total + 8 * c1.size)))
            todo = [(r, min(r + step, c1.size)) for r in range(0, c1.size, step)]
        while todo:
            r0, r1 = todo.pop(0)
            n = h.dip_block_count(c1[r0:r1], (L1, M1, p1), c2, (L2, M2, p2), 0)
            nbytes = 24 * n + 8 * (r1 - r0 + 1) + 512
            if nbytes > cap and r1 - r0 > 1:
                mid = (r0 + r1) // 2
                todo[:0] = [(r0, mid), (mid, r1)]
                continue
            out.append(dict(kind="dip", block=i1, block2=i2, r0=r0, r1=r1, rows=r1 - r0,
                            nnz=int(n), bytes=int(nbytes), owner=0))
        return out

    @staticmethod
    def _chunks(units, n):
        total = sum(u["bytes"] for u in units)
        out, cur, acc = [], [], 0
        for u in units:
            cur.append(u)
            acc += u["bytes"]
            if acc >= total * (len(out) + 1) / n and len(out) < n - 1:
                out.append(cur)
                cur = []
        out.append(cur)
        while len(out) < n:
            out.append([])
        return out

    def chunk_bytes(self, j):
        return sum(u["bytes"] for u in self.chunks[j])

    def _layout(self, parts, a):
        """Device addresses of consecutive arrays in area a (256-byte aligned)."""
        area = self.areas[a]
        out, off = [], 0
        for nbytes in parts:
            out.append(area.data_ptr() + off)
            off += (int(nbytes) + 255) // 256 * 256
        assert off <= area.numel() * area.element_size()
        return out

    def run_chunk(self, j, timers=None):
        """Chunk j on the device; timers: dict of lists of (event, event) pairs.
        Units fill the two areas in turn on the library's stream; a consumer
        thread digests (or applies) each filled unit on the consumer handle's
        stream while the next unit fills; the call returns when both are
        done."""
        import queue
        import threading
        torch, h = self.torch, self.h
        ev = (lambda: torch.cuda.Event(enable_timing=True)) if timers is not None else None

        def start(stream):
            if timers is None:
                return None
            e = ev()
            e.record(stream)
            return e

        def mark(name, e0, stream):
            if timers is not None:
                e1 = ev()
                e1.record(stream)
                timers.setdefault(name, []).append((e0, e1))

        q = queue.Queue()
        free = [threading.Event(), threading.Event()]
        for f in free:
            f.set()
        err = []
        with torch.cuda.stream(self.cstream):
            digest = torch.zeros((), dtype=torch.int64 if self.consume == "digest" else
                                 torch.complex128, device=self.dev)
        self.digests.setdefault(j, []).append(digest)

        def consumer():
            try:
                while True:
                    item = q.get()
                    if item is None:
                        return
                    a, n_rows, n_cols, mats, x = item
                    e0 = start(self.cstream)
                    for (nnz, P, I, D) in mats:
                        if self.consume == "mv":
                            self.hc.csr_mv_device(0, n_rows, n_cols, nnz, P, I, D, x,
                                                  self.y.data_ptr())
                            self._acc(n_rows, digest)
                        else:
                            with torch.cuda.stream(self.cstream):
                                for ptr, n in ((P, n_rows + 1), (I, nnz), (D, 2 * nnz)):
                                    digest.add_(self._words(a, ptr, n).sum())
                    mark("consume", e0, self.cstream)
                    if self.consume != "mv":
                        self.cstream.synchronize()
                    free[a].set()
            except BaseException as e:  # the producer re-raises it
                err.append(e)
                for f in free:
                    f.set()

        th = threading.Thread(target=consumer)
        th.start()
        try:
            if j == 0:
                e0 = start(self.stream)
                self.radial()
                mark("radial", e0, self.stream)
            for i, u in enumerate(self.chunks[j]):
                a = i % 2
                free[a].wait()
                if err:
                    break
                free[a].clear()
                if u["kind"] == "band":
                    L, M, par, spin, cf = self.blocks[u["block"]]
                    if u["count_first"]:
                        e0 = start(self.stream)
                        h.block_count(cf, L, True, spin)
                        mark("count", e0, self.stream)
                    r, nH, nS = u["rows"], u["nH"], u["nS"]
                    Hp, Hi, Hd, Sp, Si, Sd = self._layout([8 * (r + 1), 8 * nH, 16 * nH,
                                                           8 * (r + 1), 8 * nS, 16 * nS], a)
                    e0 = start(self.stream)
                    h.band_into(cf, L, u["n1"], u["m"], True, spin,
                                dict(index_ptr=Hp, indices=Hi, data=Hd),
                                dict(index_ptr=Sp, indices=Si, data=Sd))
                    mark("fill", e0, self.stream)
                    q.put((a, r, cf.size, [(nH, Hp, Hi, Hd), (nS, Sp, Si, Sd)],
                           self.x[u["block"]].data_ptr()))
                else:
                    L1, M1, p1, _, c1 = self.blocks[u["block"]]
                    L2, M2, p2, _, c2 = self.blocks[u["block2"]]
                    rows = c1[u["r0"]:u["r1"]]
                    e0 = start(self.stream)
                    n = h.dip_block_count(rows, (L1, M1, p1), c2, (L2, M2, p2), 0)
                    assert n == u["nnz"]
                    Dp, Di, Dd = self._layout([8 * (u["rows"] + 1), 8 * n, 16 * n], a)
                    h.dip_block_into(rows, (L1, M1, p1), c2, (L2, M2, p2), 0,
                                     dict(index_ptr=Dp, indices=Di, data=Dd))
                    mark("dipole", e0, self.stream)
                    q.put((a, u["rows"], c2.size, [(n, Dp, Di, Dd)],
                           self.x[u["block2"]].data_ptr()))
        finally:
            q.put(None)
            th.join()
        if err:
            raise err[0]

    def _acc(self, r, chunk_sum):
        with self.torch.cuda.stream(self.cstream):
            s = self.y[:r].sum()
            self.ysum += s
            chunk_sum += s

    def _words(self, a, ptr, n):
        """The n 64-bit words at device address ptr inside area a."""
        area = self.areas[a]
        off = ptr - area.data_ptr()
        assert off % 8 == 0 and 0 <= off and off + 8 * n <= area.numel() * 8
        return area.view(self.torch.int64)[off // 8:off // 8 + n]

    def digest_repeats(self):
        """(chunks made more than once, whether every repeat gave the same
        sum, bit for bit)."""
        runs = {j: [d.cpu().numpy().tobytes() for d in v] for j, v in self.digests.items()
                if len(v) > 1}
        return len(runs), all(len(set(v)) == 1 for v in runs.values())

    def e2e_units(self, h, units, host, counted):
        """Units through the C ABI on handle h with host outputs (pinned buffers
        in host); counted[0] is the block h counted last, and a band of another
        block counts its block first.  Returns (h2d bytes, d2h bytes)."""
        h2d = d2h = 0
        for u in units:
            if u["kind"] == "band":
                L, M, par, spin, cf = self.blocks[u["block"]]
                if counted[0] != u["block"]:
                    h.block_count(cf, L, True, spin)
                    h2d += cf.nbytes
                    counted[0] = u["block"]
                r, nH, nS = u["rows"], u["nH"], u["nS"]
                H = dict(index_ptr=host["ptrH"][:r + 1], indices=host["idxH"][:nH],
                         data=host["datH"][:nH])
                S = dict(index_ptr=host["ptrS"][:r + 1], indices=host["idxS"][:nS],
                         data=host["datS"][:nS])
                h.band_host_into(cf, L, u["n1"], u["m"], True, spin, H, S, host["rows"][:r])
                h2d += cf.nbytes
                d2h += 24 * (nH + nS) + 16 * (r + 1) + 8 * r
            else:
                L1, M1, p1, _, c1 = self.blocks[u["block"]]
                L2, M2, p2, _, c2 = self.blocks[u["block2"]]
                rows = c1[u["r0"]:u["r1"]]
                n = h.dip_block_count(rows, (L1, M1, p1), c2, (L2, M2, p2), 0)
                D = dict(index_ptr=host["ptrH"][:u["rows"] + 1], indices=host["idxH"][:n],
                         data=host["datH"][:n])
                self.pkg.lib().bs2e_dip_block_fill(
                    h._h, self.pkg._ptr(rows), rows.size, L1, M1, p1, self.pkg._ptr(c2), c2.size,
                    L2, M2, p2, 0, 1, self.pkg._ptr(D["index_ptr"]), self.pkg._ptr(D["indices"]),
                    self.pkg._ptr(D["data"]), 0)
                h2d += 2 * (rows.nbytes + c2.nbytes)
                d2h += 24 * n + 8 * (u["rows"] + 1)
        return h2d, d2h

    def e2e_chunk(self, j, handles, hosts):
        """Chunk j through the C ABI with host outputs, its units alternating
        between the handles (each with its own pinned host buffers), one thread
        per handle, so that one band's device-to-host copy runs beside the next
        band's fill; chunk 0 runs every handle's radial stage.  Every handle
        counts the blocks of its bands again in every chunk.  Returns (h2d
        bytes, d2h bytes)."""
        import threading
        units = self.chunks[j]
        n = len(handles)
        res, err = [(0, 0)] * n, []

        def work(i):
            try:
                h = handles[i]
                h2d = 0
                if j == 0:
                    self.radial(h)
                    h2d += h.knots.nbytes
                a, b = self.e2e_units(h, units[i::n], hosts[i], [-1])
                res[i] = (h2d + a, b)
            except BaseException as e:  # re-raised below
                err.append(e)

        th = [threading.Thread(target=work, args=(i,)) for i in range(n)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        if err:
            raise err[0]
        return sum(r[0] for r in res), sum(r[1] for r in res)

    def close(self):
        self.h.close()
        self.hc.close()


def run_large(args, rank, world):
    import torch
    pkg = _pkg()
    w = LARGE
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    areas = [torch.empty(w["area_bytes"] // 8, dtype=torch.float64, device=dev)
             for _ in range(2)]
    prec_main = args.precision
    precs = {"fp64": pkg.PREC_FP64, "mixed": pkg.PREC_MIXED}
    job = LargeJob(pkg, w, precs[prec_main], areas, rank, world, consume=args.consume)
    nc = w["n_chunks"]
    elems = rk_elements(w)
    total_bytes = sum(u["bytes"] for u in job.plan["units"])
    # warm-up
    for s in range(args.warmup):
        job.run_chunk(s % nc)
    _barrier(world)
    launches0 = job.h.launch_count
    timers = {}
    step_ev = []
    with Clocks(dev.index) as clk:
        _barrier(world)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev0.record(job.stream)
        for s in range(args.steps):
            e = torch.cuda.Event(enable_timing=True)
            job.run_chunk(s % nc, timers)
            e.record(job.stream)
            step_ev.append(e)
        torch.cuda.synchronize()
        _barrier(world)
    launches = job.h.launch_count - launches0
    t_steps = [ev0.elapsed_time(step_ev[0]) / 1e3] + [
        step_ev[i - 1].elapsed_time(step_ev[i]) / 1e3 for i in range(1, len(step_ev))]
    t_dev = _max_over_ranks(sum(t_steps), world)
    done_bytes = sum(job.chunk_bytes(s % nc) for s in range(args.steps))
    done_bytes = _sum_over_ranks(done_bytes, world)
    jobs_done = done_bytes / total_bytes
    value = elems * jobs_done / t_dev
    job_s = sum(t_steps[:nc]) if args.steps >= nc else None
    job_s = _max_over_ranks(job_s, world) if job_s is not None else None
    sums = {k: sum(a.elapsed_time(b) for a, b in v) / 1e3 for k, v in timers.items()}
    n_jobs_local = args.steps / nc
    fill_units = [u for j in range(args.steps) for u in job.chunks[j % nc] if u["kind"] == "band"]
    tile_b = 8 * tile_doubles(w)
    fill_bytes = sum(24 * (u["nH"] + u["nS"]) + 16 * (u["rows"] + 1) + tile_b * u["tiles"]
                     for u in fill_units)
    peak, peak_src = _peaks()
    achieved = fill_bytes / sums["fill"] / 1e9 if sums.get("fill") else None
    ratio = FILL_TRAFFIC_RATIO["order9_n800"][prec_main]
    per_launch = fill_bytes / max(len(fill_units), 1)
    res = {
        "metric": METRIC, "value": value, "unit": "R^k elements/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None,
        "dtype": "f64" if prec_main == "fp64" else "f64 out, f32-pair k-sum",
        "data": "synthetic (deterministic knot grid, no dataset)",
        "config": {"workload": workload_string(w), "precision": prec_main,
                   "step": "1/%d of a job: %d bands of 6 blocks and %d dipole row slices cut "
                           "into %d chunks of nearly equal CSR bytes, chunk 0 with the radial "
                           "stage" % (nc, sum(u["kind"] == "band" for u in job.plan["units"]),
                                      sum(u["kind"] == "dip" for u in job.plan["units"]), nc),
                   "rk_elements_per_job": elems, "csr_bytes_per_job": total_bytes,
                   "rows": [int(b[4].size) for b in job.blocks],
                   "nnz_H_S_per_job": sum(u.get("nH", 0) + u.get("nS", 0)
                                          for u in job.plan["units"]),
                   "nnz_dipole_per_job": sum(u.get("nnz", 0) for u in job.plan["units"]),
                   "l2": "every step writes ~%.0f GB of CSR (> L2)" % (total_bytes / nc / 1e9),
                   "consumer": ("bs2e_csr_mv of every band of H and S and slice of D with a "
                                "fixed vector, on the device" if args.consume == "mv" else
                                "64-bit wrapping sum of every word of every band of H and S "
                                "and slice of D (pointers, columns, value bit patterns), on "
                                "the device")},
        "job_s": job_s, "jobs_timed": jobs_done,
        "assembly_s_per_job": (sums.get("fill", 0) + sums.get("dipole", 0) + sums.get("count", 0))
                              / n_jobs_local,
        "radial_s": sums.get("radial", 0) / max(1, sum(1 for s in range(args.steps) if s % nc == 0)),
        "consume_s_per_job": sums.get("consume", 0) / n_jobs_local,
        "stage_s_per_job": {x: sums.get(x, 0) / n_jobs_local
                            for x in ("count", "fill", "dipole", "consume")},
        "rk_stage_elements_per_s": None,
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "k_csr_fill (band fills)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                     "traffic": ratio * per_launch if ratio else None, "peak_source": peak_src,
                     "algorithmic_bytes_per_launch": per_launch, "launches": len(fill_units),
                     "note": "achieved = (24 B per H/S entry + pointers + staged R^k tiles) / "
                             "CUDA-event time of the band-fill calls on the library stream"},
        "clocks": clk.summary(),
    }
    n_rep, same = job.digest_repeats()
    res["repeat_check"] = {"chunks_made_again": n_rep, "sums_repeat_bit_exact": same}
    if args.consume == "mv":
        res["checksum_y"] = complex(job.ysum.item()).__repr__()
    elif args.consume == "digest" and all(j in job.digests for j in range(nc)):
        res["repeat_check"]["job_digest"] = "%016x" % (
            sum(int(job.digests[j][0].item()) for j in range(nc)) & (2 ** 64 - 1))
    if res["radial_s"]:
        res["rk_stage_elements_per_s"] = elems / res["radial_s"]
    cs = CpuSample(pkg, w) if rank == 0 and world == 1 else None
    # mixed vs FP64: the other precision over one whole job, and the errors of
    # both against the oracle on rows of every block
    if not args.no_mixed and world == 1:
        other = "mixed" if prec_main == "fp64" else "fp64"
        job2 = LargeJob(pkg, w, precs[other], areas, rank, world, plan=job.plan,
                        consume=args.consume)
        job2.run_chunk(0)
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(job2.stream)
        for j in range(nc):
            job2.run_chunk(j)
        t1.record(job2.stream)
        torch.cuda.synchronize()
        t_other = t0.elapsed_time(t1) / 1e3
        res["mixed_vs_fp64"] = {
            other + "_job_s": t_other, prec_main + "_job_s": job_s,
            "mixed_speedup_vs_fp64": ((job_s / t_other) if prec_main == "fp64" else
                                      (t_other / job_s)) if job_s else None,
            "errors": _precision_sample(pkg, w, job.blocks, {prec_main: job.h, other: job2.h},
                                        cs)}
        job2.close()
        torch.cuda.empty_cache()
    if not args.no_e2e and world == 1:
        res["e2e"] = _e2e_large(job, args, elems, total_bytes)
    job.close()
    del areas
    torch.cuda.empty_cache()
    if cs is not None and not args.no_cpu_baseline:
        r = cs.run(w["cpu_frac"], seed=1)
        res["cpu_baseline"] = {k: v for k, v in r.items()
                               if k in ("value", "unit", "cores", "kind", "sample")}
    return res


FLOOR_EH = 1e-15  # entries below this (Hartree) take the term-scale measure only
CANCEL = 1e-3      # |entry| / sum of |terms| below which an entry is a cancellation


def _errors(got, ref, scale):
    """Max / RMS of |got - ref| over the term scale, and per entry over the
    entries >= FLOOR_EH whose terms do not cancel below CANCEL (those are
    reported apart)."""
    d = np.abs(got - ref)
    a = np.abs(ref)
    t = d / np.maximum(scale, 1e-300)
    ok = (a >= FLOOR_EH) & (a >= CANCEL * scale)
    canc = (a >= FLOOR_EH) & ~ok
    e = d[ok] / a[ok]
    return {"term_max": float(t.max()) if t.size else 0.0,
            "term_rms": float(np.sqrt(np.mean(t * t))) if t.size else 0.0,
            "entry_max": float(e.max()) if e.size else 0.0,
            "entry_rms": float(np.sqrt(np.mean(e * e))) if e.size else 0.0,
            "cancel_entry_max": float((d[canc] / a[canc]).max()) if canc.any() else 0.0,
            "entries": int(t.size), "entries_cancelling": int(canc.sum()),
            "entries_below_floor": int((a < FLOOR_EH).sum())}


def _precision_sample(pkg, w, blocks, handles, cs, places=3, per=8):
    """Rows of every block from each GPU path (handles: name -> Bs2e) and from
    the oracle, which assembles them from R^k tiles it builds from the knots
    (rk_tiles) and its own one-body matrices: each path against the oracle
    at both normalisations, and mixed against FP64."""
    from concurrent.futures import ThreadPoolExecutor
    O = cs.O
    jobs, need = [], set()
    for (L, M, par, spin, cf) in blocks:
        for r0 in np.linspace(0, cf.size - per, places).astype(np.int64):
            jobs.append((L, spin, cf, int(r0)))
            need |= set(zip(cf["n1"][r0:r0 + per].tolist(), cf["n2"][r0:r0 + per].tolist()))
    need = np.array(sorted(need), dtype=np.int64)
    T = O.rk_tiles(cs.t, w["k"], w["q"], w["max_k"], need, nthreads=cs.threads)
    tab = O.tile_table(w["n_b"], need)

    def oracle_rows(j):
        L, spin, cf, r0 = j
        return O.construct_block(cf, L, w["k"], w["n_b"], w["max_k"], T, cs.H1p, cs.S, True,
                                 spin, rows=(r0, r0 + per), tile_of=tab)[0]

    with ThreadPoolExecutor(max_workers=cs.threads) as ex:
        ref = list(ex.map(oracle_rows, jobs))
    got = {name: [h.block_rows(cf, L, r0, per, True, spin)[0] for (L, spin, cf, r0) in jobs]
           for name, h in handles.items()}
    for name in got:  # patterns bit-exact
        for g, r in zip(got[name], ref):
            assert np.array_equal(g["indices"], r["indices"]), name
    cat = lambda xs, key: np.concatenate([x[key] for x in xs])
    rd, sc = cat(ref, "data"), cat(ref, "scale")
    out = {"rows": len(jobs) * per, "pattern": "bit-exact against the oracle",
           "entry_floor_eh": FLOOR_EH, "cancel_below": CANCEL}
    for name in got:
        out[name + "_vs_oracle"] = _errors(cat(got[name], "data"), rd, sc)
    if "fp64" in got and "mixed" in got:
        out["mixed_vs_fp64"] = _errors(cat(got["mixed"], "data"), cat(got["fp64"], "data"), sc)
    return out


def _e2e_large(job, args, elems, total_bytes):
    import torch
    pkg, w = job.pkg, job.w
    nc = len(job.chunks)
    maxH = max([u.get("nH", u.get("nnz", 0)) for u in job.plan["units"]] + [1])
    maxS = max([u.get("nS", 0) for u in job.plan["units"]] + [1])
    maxr = max([u["rows"] for u in job.plan["units"]] + [1])
    pin = lambda n, dt: torch.empty(int(n), dtype=dt, pin_memory=True).numpy()
    mkhost = lambda: dict(ptrH=pin(maxr + 1, torch.int64), idxH=pin(maxH, torch.int64),
                          datH=pin(maxH, torch.complex128), ptrS=pin(maxr + 1, torch.int64),
                          idxS=pin(maxS, torch.int64), datS=pin(maxS, torch.complex128),
                          rows=pin(maxr, torch.int64))
    # a second handle of the same basis: the units of a chunk alternate
    # between the two, so one band's copy to the host runs beside the next
    # band's fill (the device-to-host rate caps each copy at ~190 GB/s)
    t = pkg.grids.explin_knots(w["k"], w["n_b"], w["r_max"])
    h2 = pkg.Bs2e(t, w["k"], w["q"], w["max_k"], precision=job.h.precision,
                  device=job.dev.index, stage_bytes=w["area_bytes"])
    h2.set_block_cache(0)
    handles, hosts = [job.h, h2], [mkhost(), mkhost()]
    try:
        n = max(1, min(args.e2e_steps, nc))
        job.e2e_chunk(0, handles, hosts)  # warm (first-touch of the pinned pages)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h2d = d2h = 0
        done = 0
        for j in range(n):
            a, b = job.e2e_chunk(j, handles, hosts)
            h2d += a
            d2h += b
            done += job.chunk_bytes(j)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
    finally:
        h2.close()
    return {"value": elems * (done / total_bytes) / t, "unit": "R^k elements/s",
            "h2d_bytes_per_step": int(h2d / n), "d2h_bytes_per_step": int(d2h / n),
            "steps": n, "s_per_step": t / n, "d2h_achieved_gbs": d2h / t / 1e9,
            "handles": len(handles),
            "timing": "wall clock, chunks 0..%d (chunk 0 with the radial stage of both "
                      "handles)" % (n - 1)}


# --------------------------------------------------------------------------
# GPU: the medium size, whole blocks into HBM
# --------------------------------------------------------------------------
def run_medium(args, rank, world):
    import torch
    pkg = _pkg()
    w = MEDIUM
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    precs = {"fp64": pkg.PREC_FP64, "mixed": pkg.PREC_MIXED}
    t = pkg.grids.explin_knots(w["k"], w["n_b"], w["r_max"])
    blocks = block_list(pkg, w)
    work = [pkg.basis.block_work(cf.size, len(set(zip(cf["l1"], cf["l2"]))))
            for (*_, cf) in blocks]
    mine = pkg.basis.shard_blocks(work, world, rank)
    elems = rk_elements(w)

    def make(prec):
        h = pkg.Bs2e(t, w["k"], w["q"], w["max_k"], precision=precs[prec], device=dev.index)
        h.set_block_cache(0)
        return h

    def radial(h):
        h.slater()
        h.rk()
        h.one_body(w["Z"], w["l_max"] + 1, w["cap_order"], w["cap_r0"], w["cap_eta"],
                   copy_out=False)

    h = make(args.precision)
    stream = torch.cuda.ExternalStream(h.stream, device=dev)
    radial(h)
    counts = {i: h.block_count(blocks[i][4], blocks[i][0], True, blocks[i][3]) for i in mine}
    out_dev = {}
    for i in mine:
        n = blocks[i][4].size
        ch, cs = counts[i]
        mk = lambda m, dt: torch.empty(max(int(m), 1), dtype=dt, device=dev)
        out_dev[i] = (dict(index_ptr=mk(n + 1, torch.int64), indices=mk(ch, torch.int64),
                           data=mk(ch, torch.complex128)),
                      dict(index_ptr=mk(n + 1, torch.int64), indices=mk(cs, torch.int64),
                           data=mk(cs, torch.complex128)))
    ptrs = {i: ({x: v.data_ptr() for x, v in a.items()}, {x: v.data_ptr() for x, v in b.items()})
            for i, (a, b) in out_dev.items()}
    tile_b = 8 * tile_doubles(w)
    n_tiles = sum(np.unique(blocks[i][4]["n1"] * 100000 + blocks[i][4]["n2"]).size for i in mine)
    fill_bytes = 24 * sum(a + b for a, b in counts.values()) + n_tiles * tile_b

    def step(hh, pp, timers=None):
        e = lambda: torch.cuda.Event(enable_timing=True)
        if timers is not None:
            r0 = e()
            r0.record(stream)
        radial(hh)
        if timers is not None:
            r1 = e()
            r1.record(stream)
            timers.setdefault("radial", []).append((r0, r1))
        for i in mine:
            L, M, par, spin, cf = blocks[i]
            hh.block_count(cf, L, True, spin)  # the count pass (no block cache)
            if timers is not None:
                f0 = e()
                f0.record(stream)
            hh.block_fill_into(cf, L, True, spin, pp[i][0], pp[i][1], on_device=True)
            if timers is not None:
                f1 = e()
                f1.record(stream)
                timers.setdefault("fill", []).append((f0, f1))

    for _ in range(args.warmup):
        step(h, ptrs)
    _barrier(world)
    launches0 = h.launch_count
    timers = {}
    with Clocks(dev.index) as clk:
        _barrier(world)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            step(h, ptrs, timers)
        ev1.record(stream)
        torch.cuda.synchronize()
        _barrier(world)
    launches = h.launch_count - launches0
    t_dev = _max_over_ranks(ev0.elapsed_time(ev1) / 1e3, world)
    sums = {k: sum(a.elapsed_time(b) for a, b in v) / 1e3 for k, v in timers.items()}
    value = elems * args.steps / t_dev
    peak, peak_src = _peaks()
    achieved = fill_bytes * args.steps / sums["fill"] / 1e9 if sums.get("fill") else None
    ratio = FILL_TRAFFIC_RATIO["order7_n200"][args.precision]
    res = {
        "metric": METRIC, "value": value, "unit": "R^k elements/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f64 out, f32-pair k-sum",
        "data": "synthetic (deterministic knot grid, no dataset)",
        "config": {"workload": workload_string(w), "precision": args.precision,
                   "blocks_this_rank": mine, "rk_elements_per_step": elems,
                   "nnz_H_S": int(sum(a + b for a, b in counts.values())),
                   "l2": "every step writes %.1f GB of CSR (> L2)" %
                         (24 * sum(a + b for a, b in counts.values()) / 1e9)},
        "assembly_s": t_dev / args.steps - sums.get("radial", 0) / args.steps,
        "radial_s": sums.get("radial", 0) / args.steps,
        "rk_stage_elements_per_s": elems / (sums["radial"] / args.steps) if sums.get("radial") else None,
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "k_csr_fill", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                     "traffic": ratio * fill_bytes / max(len(mine), 1), "peak_source": peak_src,
                     "algorithmic_bytes_per_launch": fill_bytes / max(len(mine), 1),
                     "launches_per_step": len(mine), "fill_s_per_step": sums.get("fill", 0) / args.steps},
        "clocks": clk.summary(),
    }
    cs = CpuSample(pkg, w) if rank == 0 and world == 1 else None
    if not args.no_mixed and world == 1:
        other = "mixed" if args.precision == "fp64" else "fp64"
        h2 = make(other)
        for _ in range(2):
            step(h2, ptrs)
        torch.cuda.synchronize()
        s2 = torch.cuda.ExternalStream(h2.stream, device=dev)
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(s2)
        n2 = max(2, min(args.steps, 5))
        for _ in range(n2):
            step(h2, ptrs)
        a1.record(s2)
        torch.cuda.synchronize()
        t2 = a0.elapsed_time(a1) / 1e3 / n2
        res["mixed_vs_fp64"] = {other + "_ms_per_step": 1e3 * t2,
                                args.precision + "_ms_per_step": 1e3 * t_dev / args.steps,
                                "mixed_speedup_vs_fp64": (t_dev / args.steps / t2)
                                if args.precision == "fp64" else (t2 / (t_dev / args.steps)),
                                "errors": _precision_sample(pkg, w, blocks,
                                                            {args.precision: h, other: h2}, cs)}
        h2.close()
    if not args.no_e2e and world == 1:
        del out_dev
        torch.cuda.empty_cache()
        res["e2e"] = _e2e_medium(h, pkg, w, blocks, mine, counts, args, elems, t, radial)
    h.close()
    if cs is not None and not args.no_cpu_baseline:
        r = cs.run(w["cpu_frac"], seed=1)
        res["cpu_baseline"] = {k: v for k, v in r.items()
                               if k in ("value", "unit", "cores", "kind", "sample")}
    return res


def _e2e_medium(h, pkg, w, blocks, mine, counts, args, elems, t, radial):
    import torch
    host = {}
    for i in mine:
        n = blocks[i][4].size
        ch, cs = counts[i]
        mk = lambda m, dt: torch.empty(max(int(m), 1), dtype=dt, pin_memory=True).numpy()
        host[i] = (dict(index_ptr=mk(n + 1, torch.int64), indices=mk(ch, torch.int64),
                        data=mk(ch, torch.complex128)),
                   dict(index_ptr=mk(n + 1, torch.int64), indices=mk(cs, torch.int64),
                        data=mk(cs, torch.complex128)))
    pinned_cfg = {i: torch.from_numpy(blocks[i][4].view(np.int64).copy()).pin_memory().numpy()
                  .view(pkg.CONFIG_DTYPE) for i in mine}
    h2d = t.nbytes + sum(c.nbytes for c in pinned_cfg.values())
    d2h = sum(sum(a.nbytes for a in H.values()) + sum(a.nbytes for a in S.values())
              for H, S in host.values())

    def step():
        radial(h)
        for i in mine:
            L, M, par, spin, _ = blocks[i]
            h.block_count(pinned_cfg[i], L, True, spin)
            h.block_fill_into(pinned_cfg[i], L, True, spin, host[i][0], host[i][1],
                              on_device=False)

    n = max(1, min(args.steps, args.e2e_steps))
    step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(n):
        step()
    torch.cuda.synchronize()
    te = (time.perf_counter() - t0) / n
    return {"value": elems / te, "unit": "R^k elements/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "s_per_step": te, "steps": n,
            "d2h_achieved_gbs": d2h / te / 1e9}


# --------------------------------------------------------------------------
# small cases for ncu, the ragged batch and the mat-vec
# --------------------------------------------------------------------------
def profile_band(args):
    """One band fill of the large form's method (order 9, q=12, k=0..20,
    l_max=10: 48.5 KB R^k tiles) on N = --profile-nb splines (r_max = N):
    block --profile-band, n1 = N/2 and N/2+1, a few GB of CSR (above L2).
    With N=200 the R^k store is 1.9 GB: the small case for ncu captures of
    k_csr_fill in band mode."""
    import torch
    pkg = _pkg()
    w = dict(LARGE, n_b=args.profile_nb, r_max=float(args.profile_nb))
    prec = pkg.PREC_MIXED if args.precision == "mixed" else pkg.PREC_FP64
    t = pkg.grids.explin_knots(w["k"], w["n_b"], w["r_max"])
    L, M, par, spin, cf = block_list(pkg, w)[args.profile_band]
    with pkg.Bs2e(t, w["k"], w["q"], w["max_k"], precision=prec) as h:
        h.slater()
        h.rk()
        h.one_body(w["Z"], w["l_max"] + 1, w["cap_order"], w["cap_r0"], w["cap_eta"],
                   copy_out=False)
        a, m = w["n_b"] // 2, 2
        r, nh, ns = h.band_count(cf, L, a, m, True, spin)
        dev = torch.device("cuda", 0)
        mk = lambda n, dt: torch.empty(max(int(n), 1), dtype=dt, device=dev)
        H = dict(index_ptr=mk(r + 1, torch.int64), indices=mk(nh, torch.int64),
                 data=mk(nh, torch.complex128))
        S = dict(index_ptr=mk(r + 1, torch.int64), indices=mk(ns, torch.int64),
                 data=mk(ns, torch.complex128))
        torch.cuda.synchronize()
        h.band_into(cf, L, a, m, True, spin, {x: v.data_ptr() for x, v in H.items()},
                    {x: v.data_ptr() for x, v in S.items()})
        h.synchronize()
        tiles = np.unique(cf["n1"][(cf["n1"] >= a) & (cf["n1"] < a + m)].astype(np.int64) * 1000 +
                          cf["n2"][(cf["n1"] >= a) & (cf["n1"] < a + m)]).size
        print(json.dumps({"profile_band": args.profile_band, "L": L, "n1": [a, a + m - 1],
                          "rows": int(r), "nnz_H": nh, "nnz_S": ns,
                          "algorithmic_bytes": 24 * (nh + ns) + 16 * (r + 1) +
                          8 * tile_doubles(w) * tiles, "tiles": int(tiles)}))


def profile_dip(args):
    """One dipole row slice of the large form's method (order 9, q=12,
    l_max=10, length gauge) on N = --profile-nb splines (r_max = N): rows of
    singlet block --profile-dip against block --profile-dip + 1, taken from the
    middle of the block until ~160e6 entries (~3.9 GB of CSR, above L2): the
    small case for ncu captures of k_dip_fill."""
    import torch
    pkg = _pkg()
    w = dict(LARGE, n_b=args.profile_nb, r_max=float(args.profile_nb))
    t = pkg.grids.explin_knots(w["k"], w["n_b"], w["r_max"])
    blocks = block_list(pkg, w)
    (L1, M1, p1, _, c1), (L2, M2, p2, _, c2) = blocks[args.profile_dip], blocks[args.profile_dip + 1]
    with pkg.Bs2e(t, w["k"], w["q"], w["max_k"]) as h:
        h.slater()
        h.one_body(w["Z"], w["l_max"] + 1, w["cap_order"], w["cap_r0"], w["cap_eta"],
                   copy_out=False)
        h.radial_dipole(0, copy_out=False)
        s1, s2 = (L1, M1, p1), (L2, M2, p2)
        per_row = h.dip_block_count(c1, s1, c2, s2, 0) / max(c1.size, 1)
        n_rows = int(min(c1.size, max(1, 160e6 / max(per_row, 1.0))))
        r0 = (c1.size - n_rows) // 2
        rows = c1[r0:r0 + n_rows]
        n = h.dip_block_count(rows, s1, c2, s2, 0)
        dev = torch.device("cuda", 0)
        mk = lambda m, dt: torch.empty(max(int(m), 1), dtype=dt, device=dev)
        D = dict(index_ptr=mk(n_rows + 1, torch.int64), indices=mk(n, torch.int64),
                 data=mk(n, torch.complex128))
        torch.cuda.synchronize()
        h.dip_block_into(rows, s1, c2, s2, 0, {x: v.data_ptr() for x, v in D.items()})
        h.synchronize()
        print(json.dumps({"profile_dip": [args.profile_dip, args.profile_dip + 1],
                          "L": [L1, L2], "rows": [int(r0), int(r0 + n_rows)], "nnz": int(n),
                          "algorithmic_bytes": 24 * n + 8 * (n_rows + 1)}))


def profile_block(args):
    """Small case for ncu: one radial pass, then count + fill of one block of
    the medium size into device buffers (block 0: 117,620 rows, ~2.9 GB)."""
    import torch
    pkg = _pkg()
    w = MEDIUM
    prec = pkg.PREC_MIXED if args.precision == "mixed" else pkg.PREC_FP64
    t = pkg.grids.explin_knots(w["k"], w["n_b"], w["r_max"])
    L, M, par, spin, cf = block_list(pkg, w)[args.profile_block]
    with pkg.Bs2e(t, w["k"], w["q"], w["max_k"], precision=prec) as h:
        h.slater()
        h.rk()
        h.one_body(w["Z"], w["l_max"] + 1, w["cap_order"], w["cap_r0"], w["cap_eta"],
                   copy_out=False)
        ch, cs = h.block_count(cf, L, True, spin)
        n = cf.size
        dev = torch.device("cuda", 0)
        mk = lambda m, dt: torch.empty(max(int(m), 1), dtype=dt, device=dev)
        Hd = dict(index_ptr=mk(n + 1, torch.int64), indices=mk(ch, torch.int64),
                  data=mk(ch, torch.complex128))
        Sd = dict(index_ptr=mk(n + 1, torch.int64), indices=mk(cs, torch.int64),
                  data=mk(cs, torch.complex128))
        torch.cuda.synchronize()
        h.block_fill_into(cf, L, True, spin, {x: v.data_ptr() for x, v in Hd.items()},
                          {x: v.data_ptr() for x, v in Sd.items()}, on_device=True)
        h.synchronize()
        if args.profile_mv:
            # one y = H x of the block just filled (2.7 GB of CSR read)
            x = torch.randn(n, dtype=torch.complex128, device=dev)
            y = torch.empty(n, dtype=torch.complex128, device=dev)
            torch.cuda.synchronize()
            h.csr_mv_device(0, n, n, ch, Hd["index_ptr"].data_ptr(), Hd["indices"].data_ptr(),
                            Hd["data"].data_ptr(), x.data_ptr(), y.data_ptr())
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


def run_matvec(args):
    """CSR_mv / CSR_mv_sym (bs2e_csr_mv on device pointers) over the H blocks of
    the medium size, assembled into HBM by the library: achieved GB/s of the
    mat-vec kernel against the measured copy bandwidth."""
    import torch
    pkg = _pkg()
    w = MEDIUM
    dev = torch.device("cuda", 0)
    prec = pkg.PREC_MIXED if args.precision == "mixed" else pkg.PREC_FP64
    t = pkg.grids.explin_knots(w["k"], w["n_b"], w["r_max"])
    blocks = block_list(pkg, w)
    res = {}
    with pkg.Bs2e(t, w["k"], w["q"], w["max_k"], precision=prec) as h:
        h.slater()
        h.rk()
        h.one_body(w["Z"], w["l_max"] + 1, w["cap_order"], w["cap_r0"], w["cap_eta"],
                   copy_out=False)
        stream = torch.cuda.ExternalStream(h.stream, device=dev)
        for op, full, name in ((0, True, "csr_mv"), (2, False, "csr_mv_sym")):
            t_ms, nbytes, nnz_all, cplx_all = 0.0, 0, 0, 0.0
            for (L, M, par, spin, cf) in blocks[:4]:
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
            "config": {"workload": "order 7, N=200, r_max=200, q=10, k=0..10, l_max=5, "
                                   "L=0..3 singlet", "precision_of_blocks": args.precision},
            "steps": args.steps, "warmup": args.warmup}


# --------------------------------------------------------------------------
# ranks
# --------------------------------------------------------------------------
def _barrier(world):
    import torch
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _sum_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def run_reference(args):
    """The reference's algorithm on the host cores (the oracle port, all host
    threads), same workload, metric and unit: each step is the CPU sample of
    the job described in CpuSample; ms_per_step is the measured time of that
    sample and value the sample's fraction of the job's R^k elements per
    second of it."""
    pkg = _pkg()
    w = WORKLOADS[args.workload]
    cs = CpuSample(pkg, w)
    for i in range(args.warmup):
        cs.run(w["cpu_frac"] / 8, seed=100 + i)
    vals, ts = [], []
    last = None
    for i in range(args.steps):
        last = cs.run(w["cpu_frac"], seed=1 + i)
        vals.append(last["value"])
        ts.append(last["t_s"])
    v = sum(w["cpu_frac"] * rk_elements(w) for _ in ts) / sum(ts)
    return {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "R^k elements/s",
        "n_gpus": args.gpus, "gpus_used": 0,  # the run's N; the arm itself runs on host cores
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(ts),
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (deterministic knot grid, no dataset)",
        "config": {"workload": workload_string(w),
                   "step": "the oracle on fraction f=%.3g of every stage of one job" %
                           w["cpu_frac"]},
        "full_job_s_extrapolated": statistics.mean(ts) / w["cpu_frac"],
        "cpu_baseline": {"value": v, "unit": "R^k elements/s", "cores": last["cores"],
                         "kind": "port", "sample": last["sample"]},
        "e2e": {"value": v, "unit": "R^k elements/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--consume", default="mv", choices=["mv", "digest"])
    ap.add_argument("--profile-block", type=int, default=None)
    ap.add_argument("--profile-band", type=int, default=None)
    ap.add_argument("--profile-nb", type=int, default=200)
    ap.add_argument("--profile-mv", action="store_true")
    ap.add_argument("--profile-dip", type=int, default=None)
    ap.add_argument("--workload", default="order9_n800",
                    choices=["order9_n800", "order7_n200", "batch", "matvec"])
    args = ap.parse_args()
    if args.profile_block is not None:
        profile_block(args)
        return
    if args.profile_band is not None:
        profile_band(args)
        return
    if args.profile_dip is not None:
        profile_dip(args)
        return
    if args.workload == "batch":
        print(json.dumps(run_batch(args)), flush=True)
        return
    if args.workload == "matvec":
        print(json.dumps(run_matvec(args)), flush=True)
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
    res = run_large(args, rank, world) if args.workload == "order9_n800" else \
        run_medium(args, rank, world)
    if rank == 0:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
