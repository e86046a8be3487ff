r"""Benchmark of the CI hot path on GB300: Davidson seconds per root (mixed
FP32/FP64 and plain FP64) and SpMV HBM bandwidth, on the 12-orbital,
5 alpha + 5 beta FCI workload (627,264 determinants, 1.08e9 stored nonzeros)
with seeded synthetic integrals.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on rank 0.  A step is one lowest-4-roots mixed-precision solve
on the CSR already resident in HBM (`value`, s/root, lower is better); `e2e`
is the same metric through the public API with host buffers (sparse_op build
from host integrals + solve + eigenvectors back to the host).  The matrix
(8.6 GB of FP32 values + int32 columns) is far larger than L2, so every SpMM
streams it from HBM; no L2 flush is needed.

--impl reference times the reference algorithm on the host cores: the CPU
oracle's CSR build (a restatement of pyci/src/sparseop.cpp, all threads) and
ARPACK's implicitly restarted Lanczos (the algorithm of Spectra's
SymEigsSolver) on the oracle's threaded self-adjoint SpMV.
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
sys.path.insert(0, ROOT)

WORKLOADS = {
    "fci8": {"workload": "FullCI nbasis=8 4a4b (4900 dets), lowest root, synthetic seeded integrals",
             "wfn": "fullci", "nbasis": 8, "nocc_up": 4, "nocc_dn": 4, "nroot": 1, "seed": 1001,
             "golden": "fci_8_4_4",
             "metric": "Davidson s/root at <=1 uHa (FP32-mixed), FCI(8o,8e) lowest root; SpMV GB/s"},
    "doci24": {"workload": "DOCI nbasis=24 6 pairs (134596 dets), lowest root, tol 1e-8, synthetic seeded integrals",
               "wfn": "doci", "nbasis": 24, "nocc_up": 6, "nocc_dn": 6, "nroot": 1, "seed": 1002, "tol": 1e-8,
               "golden": "doci_24_6",
               "metric": "Davidson s/root at <=1 uHa (FP32-mixed), DOCI(24o, 6 pairs) lowest root; SpMV GB/s"},
    "fci12": {"workload": "FullCI nbasis=12 5a5b (627264 dets), lowest 4 roots, synthetic seeded integrals",
              "wfn": "fullci", "nbasis": 12, "nocc_up": 5, "nocc_dn": 5, "nroot": 4, "seed": 1003,
              "golden": "fci_12_5_5",
              "metric": "Davidson s/root at <=1 uHa (FP32-mixed), FCI(12o,10e) 4 roots; SpMV HBM GB/s"},
    "doci32": {"workload": "DOCI nbasis=32 8 pairs (10518300 dets), lowest 4 roots, synthetic seeded integrals",
               "wfn": "doci", "nbasis": 32, "nocc_up": 8, "nocc_dn": 8, "nroot": 4, "seed": 1004,
               "golden": "doci_32_8",
               "metric": "Davidson s/root at <=1 uHa (FP32-mixed), DOCI(32o, 8 pairs) 4 roots; SpMV HBM GB/s"},
}
WORKLOAD = WORKLOADS["fci12"]
METRIC = WORKLOAD["metric"]
# DRAM bytes moved per algorithmic byte by the FP32 k = 4 SpMM, per kernel
# form, from one ncu capture of the same kernel on the 11-orbital 5a5b FullCI
# operator (SELL-32: 2.1617 GB moved for 2.1621 GB algorithmic).  Both
# operators stream the matrix once per launch with the x block in L2, so
# traffic scales with the entries processed.
FORM_NAMES = {-1: "untuned", 0: "csr", 1: "sell32", 2: "implicit"}
KERNEL_NAMES = {-1: "untuned", 0: "CSR spmm_kernel tile", 1: "spmm_sell_kernel (SELL-32)",
                2: "fcix_spmm_kernel (implicit columns, values only)"}
TRAFFIC_PER_ALGORITHMIC_BYTE = {-1: 1.0, 0: 1.024, 1: 1.000, 2: 1.000}
DOCI_IMPLICIT_KERNEL = "docx_spmm_kernel (columns from each row's occupation, values from the pair integrals)"
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum, one ncu pass) of
# one FP32 k = 4 launch of the dominant kernel, measured on the benchmark
# operators themselves: the implicit-column product of the 12-orbital 5a5b
# FullCI operator (4,370,828,288 + 5,650,176) and the implicit product of the
# 32-orbital 8-pair DOCI operator (1,480,721,664 + 164,033,792: x, 168 MB,
# re-read from DRAM, 86 % L2 hits).
MEASURED_TRAFFIC = {("fci12", 2): 4376478464, ("doci32", 2): 1644755456}
# The implicit-column form streams padded packets (beta strings padded to a
# multiple of 32 rows per alpha string, row sections to multiples of 4
# entries); on the 11-orbital 5a5b operator ncu measured 1.001 DRAM bytes per
# byte of padded values + x + y (1.1581 GB for 1.1564 GB).
IMPLICIT_TRAFFIC_PER_PADDED_BYTE = 1.001


def implicit_padded_bytes(nb, na, nbeta_occ, k):
    r"""Bytes of one implicit-column FP32 product at width k: padded value
    packets plus x read once and y written once."""
    from math import comb
    nalpha, nbeta = comb(nb, na), comb(nb, nbeta_occ)
    nbp = (nbeta + 31) // 32 * 32

    def up4(v):
        return (v + 3) // 4 * 4

    sa, sb = na * (nb - na), nbeta_occ * (nb - nbeta_occ)
    da = comb(na, 2) * comb(nb - na, 2)
    db = comb(nbeta_occ, 2) * comb(nb - nbeta_occ, 2)
    row = up4(1 + sb + db) + sa * up4(1 + sb) + up4(da)
    return nalpha * nbp * row * 4 + 2 * nalpha * nbeta * k * 4
TOL = 1.0e-6  # residual <= 1e-6 * |E| (~1e-5 Ha): eigenvalues converge quadratically, well inside 1 uHa


def dist_init(args, backend=None):
    r"""One process per GPU (torchrun's env vars); returns (world, rank, local).
    The path shards into independent replicas or problems, so the only
    collectives are the timing barrier and the max over ranks."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        if backend is None:
            backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def shard(items, rank, world):
    r"""Round-robin share of `items` for `rank` (independent problems, no exchange)."""
    return [x for i, x in enumerate(items) if i % world == rank]


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    r"""nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
                for name, v in zip(names, r[4:8]):
                    if v.lower() == "active":
                        reasons.add(name)
            except (ValueError, IndexError):
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def reference_eigenvalues():
    try:
        with open(os.path.join(ROOT, "tests", "golden", "digests.json")) as f:
            w = json.load(f)["workloads"].get(WORKLOAD["golden"])
        return None if w is None else np.array(w["eigenvalues"])
    except OSError:
        return None


def load_synth():
    r"""The synthetic-integral recipe (pyci_gb300/synth.py, pure numpy) loaded
    by path, so that the CPU arm never imports the pyci_gb300 package (whose
    __init__ loads the GPU library and the host module)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("pyci_gb300_synth", os.path.join(ROOT, "pyci_gb300", "synth.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.synthetic_integrals


def load_oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    return O


def workload_config(ndet, stored, size, world):
    r"""The `config` object of both arms: the workload, its sizes (stored =
    both triangles, as the GPU keeps them; reference = the reference's lower
    layout), roots, tolerance, L2 note and parallelism.  The L2 note names
    what a step streams: the FP32 values of the implicit-column FullCI form
    (none per entry for the implicit DOCI form) and the eigensolver's FP32
    subspace (V and H V, 16 vectors per root)."""
    values = 0 if WORKLOAD["wfn"] == "doci" else stored * 4
    subspace = 2 * 16 * WORKLOAD["nroot"] * ndet * 4
    streamed = ("no per-entry bytes (implicit DOCI form)" if values == 0
                else "%.2f GB of FP32 values per product" % (values / 1e9))
    big = max(values, subspace) > 2**28
    l2 = "%s; subspace %.2f GB; %s" % (streamed, subspace / 1e9,
                                       "> 129 MB L2, no flush needed" if big
                                       else "fits in the 129 MB L2: figures are L2-resident")
    return {"workload": WORKLOAD["workload"], "ndet": int(ndet), "nnz_stored": int(stored),
            "nnz_reference": int(size), "roots": WORKLOAD["nroot"], "tol": WORKLOAD.get("tol", TOL),
            "l2": l2, "parallelism": "replicas" if world > 1 else "single GPU"}


def cpu_problem(O):
    synthetic_integrals = load_synth()
    ecore, one, two = synthetic_integrals(WORKLOAD["nbasis"], WORKLOAD["seed"])
    kind = O.FULLCI if WORKLOAD["wfn"] == "fullci" else O.DOCI
    return kind, ecore, one, two


def arpack(O, csr, nthreads, counter=None):
    r"""ARPACK's implicitly restarted Lanczos (the algorithm of Spectra's
    SymEigsSolver, with the reference's ncv = max(2 n + 1, 20)) on the
    oracle's threaded self-adjoint SpMV, from a seeded random start (the
    reference's solver starts from a random vector)."""
    import scipy.sparse.linalg as spl
    n = csr[2].shape[0] - 1
    nroot = WORKLOAD["nroot"]

    def mv(x):
        if counter is not None:
            counter[0] += 1
        return O.spmv(*csr, np.ravel(x), nthreads=nthreads)

    op = spl.LinearOperator((n, n), matvec=mv, dtype=np.float64)
    evals = spl.eigsh(op, k=nroot, which="SA", tol=WORKLOAD.get("tol", TOL), return_eigenvectors=False,
                      v0=np.random.default_rng(7).standard_normal(n), ncv=max(2 * nroot + 1, 20))
    return np.sort(evals)


def cpu_solve(nthreads):
    r"""One full CPU solve of the workload with the oracle; returns
    (seconds, build seconds, eigenvalues)."""
    O = load_oracle()
    kind, ecore, one, two = cpu_problem(O)
    t0 = time.perf_counter()
    dets = O.all_dets(kind, WORKLOAD["nbasis"], WORKLOAD["nocc_up"], WORKLOAD["nocc_dn"])
    csr = O.build_csr(kind, WORKLOAD["nbasis"], WORKLOAD["nocc_up"], WORKLOAD["nocc_dn"], dets, one, two,
                      nthreads=nthreads)
    t1 = time.perf_counter()
    evals = arpack(O, csr, nthreads)
    t2 = time.perf_counter()
    return t2 - t0, t1 - t0, evals + ecore


def run_reference(args, world, rank):
    r"""The reference algorithm on the host cores, in bounded samples.

    Preparation (untimed): the oracle builds the whole operator once and
    ARPACK solves it once, which gives the solve's SpMV count M.  The work of
    one full solve is then cut into K equal samples, one per timed step:
    step s builds rows [s N / K, (s + 1) N / K) of the operator (count and
    fill passes, all threads) and applies the whole operator M / K times.
    The K steps together are the build plus every product of one solve, so
    value = (sum of the K step times) / roots.  ARPACK's own dense work
    between products is not in the samples (it favours the CPU figure).
    Only rank 0 works; the other ranks exit without work."""
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    O = load_oracle()
    kind, ecore, one, two = cpu_problem(O)
    nb, nu, nd = WORKLOAD["nbasis"], WORKLOAD["nocc_up"], WORKLOAD["nocc_dn"]
    nroot = WORKLOAD["nroot"]
    dets = O.all_dets(kind, nb, nu, nd)
    n = dets.shape[0]
    t0 = time.perf_counter()
    csr = O.build_csr(kind, nb, nu, nd, dets, one, two, nthreads=nthreads)
    t_build_full = time.perf_counter() - t0
    size = int(csr[2][-1])
    count = [0]
    t0 = time.perf_counter()
    evals = arpack(O, csr, nthreads, count)
    t_solve_full = time.perf_counter() - t0
    nmv = count[0]
    hvw = O.senzero(one, two)
    x = np.random.default_rng(11).standard_normal(n)
    K = max(1, args.steps)

    def sample(s):
        r0, r1 = s * n // K, (s + 1) * n // K
        O.build_csr_rows(kind, nb, nu, nd, dets, one, two, r0, r1, nthreads=nthreads, h_v_w=hvw)
        for _ in range(nmv * (s + 1) // K - nmv * s // K):
            O.spmv(*csr, x, nthreads=nthreads)

    for w in range(args.warmup):
        sample(w % K)
    times = []
    for s in range(K):
        t0 = time.perf_counter()
        sample(s)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    spr = total / nroot
    line = {"impl": "reference", "metric": METRIC, "value": spr, "unit": "s/root", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / K,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic seeded integrals (seed %d)" % WORKLOAD["seed"],
            "config": workload_config(n, 2 * size - n, size, world),
            "cpu_baseline": {"value": spr, "unit": "s/root", "cores": nthreads, "kind": "port",
                             "sample": "one full solve cut into %d samples, one per step: step s builds 1/%d of the "
                                       "rows with the C oracle (restating pyci/src/sparseop.cpp, %d threads) and "
                                       "applies the whole operator %d/%d of the %d times ARPACK's implicitly "
                                       "restarted Lanczos needed (tol %.0e); value = sum of the step times / %d "
                                       "roots" % (K, K, nthreads, 1, K, nmv, WORKLOAD.get("tol", TOL), nroot)},
            "e2e": {"value": spr, "unit": "s/root", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "preparation": {"full_build_seconds": t_build_full, "full_arpack_seconds": t_solve_full,
                            "arpack_products": nmv, "eigenvalues": list(evals + ecore)}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch
    import pyci_gb300 as pyci
    from pyci_gb300 import capi
    from pyci_gb300.synth import synthetic_integrals

    torch.cuda.set_device(local)
    os.environ["PYCI_GPU_DEVICE"] = str(local)
    lib = capi.lib()
    ctx = capi.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    nb, nu, nd, nroot = WORKLOAD["nbasis"], WORKLOAD["nocc_up"], WORKLOAD["nocc_dn"], WORKLOAD["nroot"]
    ecore, one, two = synthetic_integrals(nb, WORKLOAD["seed"])
    from math import comb
    fci = WORKLOAD["wfn"] == "fullci"
    kind = capi.WFN_FULLCI if fci else capi.WFN_DOCI
    ndet = comb(nb, nu) * (comb(nb, nd) if fci else 1)

    # ---- resident CSR, built once (build time reported separately)
    t0 = time.perf_counter()
    csr = capi.Csr(ctx, kind, nb, nu, nd, None, one, two, flags=capi.BUILD_FULL_COLEX, ndet=ndet)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    nrow, ncol, size, stored = csr.shape()
    csr.prepare_mixed()

    tol = WORKLOAD.get("tol", TOL)

    def solve(mode):
        # Eigenvalues only: the device-resident metric does not copy the
        # eigenvectors out (the e2e number below does).
        return csr.solve(n=nroot, tol=tol, ecore=ecore, mode=mode, evecs=False)

    for _ in range(args.warmup):
        solve(capi.SOLVE_MIXED)
    ref = reference_eigenvalues()

    # ---- timed: mixed-precision solves on the resident CSR
    barrier(world)
    torch.cuda.synchronize()
    launches0 = lib.pyci_gpu_kernel_launches()
    with ClockSampler(local) as clocks:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        stats = []
        evals_mixed = None
        ev0.record(stream)
        for _ in range(args.steps):
            evals_mixed, _, st = solve(capi.SOLVE_MIXED)
            stats.append(st)
        ev1.record(stream)
        ev1.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    launches = lib.pyci_gpu_kernel_launches() - launches0
    ms_total = max_over_ranks(ev0.elapsed_time(ev1), world)
    ms_step = ms_total / args.steps
    value = ms_step / 1e3 / (nroot * world)

    # ---- FP64 path on the same resident operator (for the mixed-vs-FP64
    # speedup): FP64 vectors, Gram products and Rayleigh-Ritz; products
    # FP64-accurate in double-float arithmetic on the exact high/low split.
    # The same solve with FP64-arithmetic products is timed beside it.
    def time_solves(mode, reps):
        solve(mode)
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(reps):
            ev_, _, st_ = solve(mode)
        f1.record(stream)
        f1.synchronize()
        return f0.elapsed_time(f1) / reps / 1e3 / nroot, ev_, st_

    nf = max(1, min(2, args.steps))
    fp64_spr, evals64, st64 = time_solves(capi.SOLVE_FP64, nf)
    os.environ["PYCI_GPU_FP64_PRODUCT"] = "native"
    try:
        fp64n_spr, evals64n, st64n = time_solves(capi.SOLVE_FP64, 1)
    finally:
        os.environ.pop("PYCI_GPU_FP64_PRODUCT", None)

    # ---- SpMV / SpMM bandwidth (dominant kernel), events on the launch stream
    N = nrow
    x32 = torch.randn((N, nroot), dtype=torch.float32, device="cuda")
    y32 = torch.empty_like(x32)
    x64 = torch.randn((N, 1), dtype=torch.float64, device="cuda")
    y64 = torch.empty_like(x64)

    def time_spmm(prec, k, x, y, reps=10):
        for _ in range(3):
            csr.spmm_device(prec, k, x.data_ptr(), y.data_ptr(), ctx.stream)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            csr.spmm_device(prec, k, x.data_ptr(), y.data_ptr(), ctx.stream)
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / reps / 1e3

    t32 = time_spmm(capi.PREC_FP32, nroot, x32, y32)
    t64 = time_spmm(capi.PREC_FP64, 1, x64, y64)
    # FP64-accurate 4-vector product in FP32 arithmetic (the refinement's and
    # the FP64 solve's product)
    xdf = torch.randn((N, 8), dtype=torch.float32, device="cuda")
    ydf = torch.empty((N, 4), dtype=torch.float64, device="cuda")
    tdf = time_spmm(capi.PREC_FP64_DF, 4, xdf, ydf)
    del xdf, ydf
    form32 = csr.product_form(capi.PREC_FP32, nroot)
    formdf = csr.product_form(capi.PREC_FP64_DF, 4)
    # Algorithmic bytes of one launch: the stored values (+ int32 columns and
    # row pointers unless the columns are implicit), x read once, y written once.
    # The implicit DOCI form stores nothing per entry: x, y and the FP64
    # diagonal are its only HBM traffic.
    if form32 == capi.FORM_IMPLICIT:
        bytes32 = (stored * 4 if fci else N * 8) + 2 * N * nroot * 4
    else:
        bytes32 = stored * (4 + 4) + (N + 1) * 8 + 2 * N * nroot * 4
    if formdf == capi.FORM_IMPLICIT:
        bytesdf = (stored * 8 if fci else N * 8) + N * (32 + 32)
    else:
        bytesdf = stored * 12 + (N + 1) * 8 + N * (32 + 32)
    bytes64 = stored * (8 + 4) + (N + 1) * 8 + 2 * N * 8
    peaks, peak_kind = measured_peaks()
    hbm = float(peaks["hbm_gbs"])
    gbs32 = bytes32 / t32 / 1e9
    gbs64 = bytes64 / t64 / 1e9
    del x32, y32, x64, y64

    # ---- end to end through the public API with host buffers
    ham = pyci.secondquant_op(ecore, one, two)
    wfn = (pyci.fullci_wfn if fci else pyci.doci_wfn)(nb, nu, nd)
    wfn.add_all_dets()
    csr.free()  # make room: the e2e path builds its own operator
    e2e_times = []
    e2e_warm = max(1, min(3, args.warmup))
    for i in range(max(1, min(5, args.steps)) + e2e_warm):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op = pyci.sparse_op(ham, wfn)
        es, cs = op.solve(n=nroot, tol=tol, mode="mixed")
        t1 = time.perf_counter()
        del op
        if i >= e2e_warm:  # the first W steps are warm-up
            e2e_times.append(t1 - t0)
    e2e_spr = max_over_ranks(statistics.median(e2e_times), world) / (nroot * world)
    h2d = one.nbytes + two.nbytes
    d2h = cs.nbytes + es.nbytes

    # ---- CPU baseline sample (rank 0 only, N = 1)
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        nthreads = os.cpu_count() or 1
        tcpu, tbuild, ev_cpu = cpu_solve(nthreads)
        cpu = {"value": tcpu / nroot, "unit": "s/root", "cores": nthreads, "kind": "port",
               "sample": "one full solve of the same workload: C oracle CSR build (%.1f s, %d threads) + "
                         "ARPACK IRL on the oracle's threaded SpMV, tol %.0e" % (tbuild, nthreads, tol)}

    if rank != 0:
        return
    # Roofline traffic: measured on this very operator where a capture
    # exists, else scaled from the 11-orbital capture of the same kernel.
    wname = next((k for k, w in WORKLOADS.items() if w is WORKLOAD), None)
    if (wname, form32) in MEASURED_TRAFFIC and nroot == 4:
        traffic = MEASURED_TRAFFIC[(wname, form32)]
        traffic_source = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the same kernel on this operator "
                          "(one pass, FP32 k=4)")
    elif fci:
        traffic = (int(IMPLICIT_TRAFFIC_PER_PADDED_BYTE * implicit_padded_bytes(nb, nu, nd, nroot))
                   if form32 == capi.FORM_IMPLICIT else int(bytes32 * TRAFFIC_PER_ALGORITHMIC_BYTE[form32]))
        traffic_source = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the same kernel on FullCI 11o 5a5b, "
                          "scaled by entries processed")
    else:
        traffic, traffic_source = None, None
    errs = None
    if ref is not None:
        errs = {"mixed_uHa": list(np.abs(np.sort(evals_mixed) - ecore - ref[:nroot]) * 1e6),
                "fp64_uHa": list(np.abs(np.sort(evals64) - ecore - ref[:nroot]) * 1e6)}
    line = {
        "metric": METRIC, "value": value, "unit": "s/root", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic seeded integrals (seed %d)" % WORKLOAD["seed"],
        "config": workload_config(N, stored, size, world),
        "fp64": {"s_per_root": fp64_spr, "iterations": st64["iterations"], "matvecs": st64["matvecs"],
                 "products": "double-float (FP32 arithmetic, FP64-accurate) on the exact high/low split"},
        "fp64_native": {"s_per_root": fp64n_spr, "iterations": st64n["iterations"], "matvecs": st64n["matvecs"],
                        "products": "FP64 arithmetic on the FP64 CSR (bound by the FP64 pipe)"},
        "speedup_mixed_vs_fp64": fp64_spr / (ms_step / 1e3 / nroot),
        "speedup_mixed_vs_fp64_native": fp64n_spr / (ms_step / 1e3 / nroot),
        "mixed": {"iterations": stats[-1]["iterations"], "matvecs": stats[-1]["matvecs"],
                  "matvecs_fp64": stats[-1]["matvecs_fp64"], "refinements": stats[-1]["refinements"],
                  "spmm_seconds": stats[-1]["seconds_spmm"], "max_residual": stats[-1]["max_residual"],
                  "host_syncs": stats[-1]["host_syncs"], "host_wait_seconds": stats[-1]["seconds_wait"],
                  "solve_seconds": stats[-1]["seconds"]},
        "error_vs_fp64_oracle": errs,
        "build_seconds": build_s,
        "spmv": {"fp32_k4_gbs": gbs32, "fp32_k4_ms": t32 * 1e3, "fp32_k4_form": FORM_NAMES[form32],
                 "fp64_k1_gbs": gbs64, "fp64_k1_ms": t64 * 1e3, "fp64_k1_frac": gbs64 / hbm,
                 "df_k4_ms": tdf * 1e3, "df_k4_gbs": bytesdf / tdf / 1e9, "df_k4_frac": bytesdf / tdf / 1e9 / hbm,
                 "df_k4_form": FORM_NAMES[formdf]},
        "roofline": {"bound": "hbm", "achieved": gbs32, "peak": hbm, "unit": "GB/s", "frac": gbs32 / hbm,
                     "traffic": traffic,
                     "traffic_source": traffic_source,
                     "peak_source": peak_kind, "peak_note": "of measured" if peak_kind == "measured" else "of fallback",
                     "kernel": "FP32 k=4 SpMM, autotuned: " + (KERNEL_NAMES[form32] if fci or form32 != capi.FORM_IMPLICIT
                                                                  else DOCI_IMPLICIT_KERNEL),
                     "algorithmic_bytes": bytes32},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_spr, "unit": "s/root", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)


def batch_problems():
    r"""The 64 uneven FullCI problems: nbasis in {8, 10, 12}, alpha = beta in
    [2, nbasis / 2], drawn from default_rng(4242); problem i uses seed 5000 + i."""
    rng = np.random.default_rng(4242)
    out = []
    for i in range(64):
        n = int(rng.choice([8, 10, 12]))
        a = int(rng.integers(2, n // 2 + 1))
        out.append((n, a, 5000 + i))
    return out


def run_batch(args, world=1, rank=0, local=0):
    r"""64 independent FCI problems, lowest 4 roots each, one batched mixed
    solve per rank.  With N ranks each GPU takes a round-robin share of the
    problems (no exchange between ranks); value = 64 / the slowest rank's time."""
    import torch
    from math import comb
    from pyci_gb300 import capi
    from pyci_gb300.synth import synthetic_integrals
    torch.cuda.set_device(local)
    ctx = capi.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    probs = shard(list(enumerate(batch_problems())), rank, world)
    ops, ecore = [], []
    t0 = time.perf_counter()
    for _, (n, a, seed) in probs:
        e, one, two = synthetic_integrals(n, seed)
        csr = capi.Csr(ctx, capi.WFN_FULLCI, n, a, a, None, one, two, flags=capi.BUILD_FULL_COLEX,
                       ndet=comb(n, a) ** 2)
        csr.prepare_mixed(drop_fp64=True)  # 12 bytes per entry: all 64 fit in HBM together
        ops.append(csr)
        ecore.append(e)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    nnz = sum(c.shape()[3] for c in ops)
    rows = sum(c.shape()[0] for c in ops)
    for _ in range(args.warmup):
        capi.batch_solve(ctx, ops, ecore, n=4, tol=TOL, mode=capi.SOLVE_MIXED)
    lib = capi.lib()
    barrier(world)
    torch.cuda.synchronize()
    launches0 = lib.pyci_gpu_kernel_launches()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        ev0.record(stream)
        for _ in range(args.steps):
            evals, st = capi.batch_solve(ctx, ops, ecore, n=4, tol=TOL, mode=capi.SOLVE_MIXED)
        ev1.record(stream)
        ev1.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    launches = (lib.pyci_gpu_kernel_launches() - launches0) // args.steps
    batch_s = max_over_ranks(ev0.elapsed_time(ev1) / 1e3 / args.steps, world)
    # One at a time, same operators, for comparison; FP64 references (high + low values).
    t0 = time.perf_counter()
    seq_iters = []
    for i, c in enumerate(ops):
        seq_iters.append(c.solve(n=4, tol=TOL, ecore=ecore[i], mode=capi.SOLVE_MIXED, evecs=False)[2]["iterations"])
    torch.cuda.synchronize()
    seq_s = max_over_ranks(time.perf_counter() - t0, world)
    err = {}
    for i, c in enumerate(ops):
        ref, _, _ = c.solve(n=4, tol=1e-9, ecore=ecore[i], mode=capi.SOLVE_FP64, evecs=False)
        err[probs[i][0]] = float(np.max(np.abs(evals[i] - ref))) * 1e6
    its = {probs[i][0]: (st["per_problem_iterations"][i], seq_iters[i]) for i in range(len(ops))}
    if world > 1:
        import torch.distributed as dist
        parts = [None] * world
        dist.all_gather_object(parts, (err, its, rows, nnz, st["iterations"]))
        err, its = {}, {}
        rows = nnz = lock = 0
        for e_, i_, r_, z_, l_ in parts:
            err.update(e_)
            its.update(i_)
            rows += r_
            nnz += z_
            lock = max(lock, l_)
        st = dict(st, iterations=lock)
    if rank != 0:
        return
    order = sorted(err)
    line = {"metric": "batched solves/s, 64 uneven FCI problems, 4 roots each (mixed)", "value": 64 / batch_s,
            "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": batch_s * 1e3, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "64 x FullCI, nbasis in {8,10,12}, alpha=beta in [2, nbasis/2], "
                                   "default_rng(4242), seeds 5000+i", "rows": rows, "nnz_stored": nnz,
                       "tol": TOL, "parallelism": "problems sharded round-robin over %d GPU(s)" % world},
            "build_seconds": build_s, "batched_seconds": batch_s, "sequential_mixed_seconds": seq_s,
            "batched_speedup_vs_sequential": seq_s / batch_s, "iterations": st["iterations"],
            "per_problem_iterations": [its[i][0] for i in order],
            "sequential_iterations": [its[i][1] for i in order],
            "max_residual_fp64": st["max_residual"], "seconds_spmm": st["seconds_spmm"],
            "max_error_uHa_vs_fp64": max(err.values()), "per_problem_error_uHa": [err[i] for i in order],
            "gpu_launches": launches, "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def run_hci(args, world=1, rank=0, local=0):
    r"""One heat-bath CI selection step (add_hci) on the 12-orbital FCI
    Hamiltonian: the wave function is every determinant of the FP64 ground
    state with |c| > 1e-4, in colex order, with those coefficients; the step
    uses eps = 1e-5.  value = seconds per step through the C ABI (host arrays
    in and out, as the reference's call); the same step of the CPU oracle
    (a serial restatement of pyci/src/hci.cpp) is the baseline, and the two
    results must be identical.  Independent replicas under torchrun."""
    import torch
    from math import comb
    from pyci_gb300 import capi
    from pyci_gb300.synth import synthetic_integrals
    torch.cuda.set_device(local)
    nb, na, nbeta, eps = 12, 5, 5, 1.0e-5
    ctx = capi.Context(local)
    ecore, one, two = synthetic_integrals(nb, 1003)
    csr = capi.Csr(ctx, capi.WFN_FULLCI, nb, na, nbeta, None, one, two, flags=capi.BUILD_FULL_COLEX,
                   ndet=comb(nb, na) * comb(nb, nbeta))
    _, vecs, _ = csr.solve(n=1, tol=1e-8, ecore=ecore, mode=capi.SOLVE_FP64)
    csr.free()
    full = ctx.add_all_dets(capi.WFN_FULLCI, nb, na, nbeta)
    keep = np.nonzero(np.abs(vecs[0]) > 1e-4)[0]
    dets, coeffs = np.ascontiguousarray(full[keep]), np.ascontiguousarray(vecs[0][keep])
    del full
    for _ in range(args.warmup):
        new = ctx.add_hci(capi.WFN_FULLCI, nb, na, nbeta, dets, coeffs, one, two, eps)
    lib = capi.lib()
    barrier(world)
    launches0 = lib.pyci_gpu_kernel_launches()
    times = []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            new = ctx.add_hci(capi.WFN_FULLCI, nb, na, nbeta, dets, coeffs, one, two, eps)
            times.append(time.perf_counter() - t0)
    launches = (lib.pyci_gpu_kernel_launches() - launches0) // args.steps
    t_gpu = max_over_ranks(statistics.median(times), world)
    if rank != 0:
        return
    line = {"metric": "heat-bath CI selection step (add_hci) seconds, FCI(12o,10e)", "value": t_gpu, "unit": "s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_gpu * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic seeded integrals (seed 1003)",
            "config": {"workload": "add_hci on FCI nbasis=12 5a5b: determinants with |c| > 1e-4 in the FP64 "
                                   "ground state, eps = 1e-5", "ndet_in": int(dets.shape[0]),
                       "added": int(new.shape[0]), "parallelism": "replicas"},
            "e2e": {"value": t_gpu, "unit": "s", "h2d_bytes_per_step": int(dets.nbytes + coeffs.nbytes + one.nbytes
                                                                           + two.nbytes),
                    "d2h_bytes_per_step": int(new.nbytes)},
            "gpu_launches": launches, "clocks": clocks.summary()}
    if not args.skip_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        t0 = time.perf_counter()
        ref = O.add_hci(O.FULLCI, nb, na, nbeta, dets, coeffs, one, two, eps)
        t_cpu = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": t_cpu, "unit": "s", "cores": 1, "kind": "port",
                                "sample": "the same step with the C oracle (serial restatement of pyci/src/hci.cpp; "
                                          "the reference's add_hci runs PYCI_NUM_THREADS = 1 threads by default)"}
        line["parity"] = "identical to the oracle" if np.array_equal(new, ref) else "MISMATCH vs the oracle"
    print(json.dumps(line), flush=True)


def run_rdm(args, world=1, rank=0, local=0):
    r"""compute_rdms of the FP64 ground state of the 10-orbital 5a5b FCI
    Hamiltonian (63,504 determinants): rdm1 [2, 10, 10] and rdm2
    [3, 10, 10, 10, 10].  value = seconds per call through the C ABI (host
    arrays in and out, as the reference's call); the same call of the CPU
    oracle (a serial restatement of pyci/src/rdm.cpp, as the reference runs it)
    is the baseline, and the arrays must agree to 1e-12.  Replicas under
    torchrun."""
    import torch
    from math import comb
    from pyci_gb300 import capi
    from pyci_gb300.synth import synthetic_integrals
    torch.cuda.set_device(local)
    nb, na, nbeta = 10, 5, 5
    ctx = capi.Context(local)
    ecore, one, two = synthetic_integrals(nb, 1000 + nb)
    ndet = comb(nb, na) * comb(nb, nbeta)
    csr = capi.Csr(ctx, capi.WFN_FULLCI, nb, na, nbeta, None, one, two, flags=capi.BUILD_FULL_COLEX, ndet=ndet)
    _, vecs, _ = csr.solve(n=1, tol=1e-8, ecore=ecore, mode=capi.SOLVE_FP64)
    csr.free()
    dets = ctx.add_all_dets(capi.WFN_FULLCI, nb, na, nbeta)
    coeffs = np.ascontiguousarray(vecs[0])
    for _ in range(args.warmup):
        r1, r2 = ctx.compute_rdms(capi.WFN_FULLCI, nb, na, nbeta, dets, coeffs)
    lib = capi.lib()
    barrier(world)
    launches0 = lib.pyci_gpu_kernel_launches()
    times = []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r1, r2 = ctx.compute_rdms(capi.WFN_FULLCI, nb, na, nbeta, dets, coeffs)
            times.append(time.perf_counter() - t0)
    launches = (lib.pyci_gpu_kernel_launches() - launches0) // args.steps
    t_gpu = max_over_ranks(statistics.median(times), world)
    if rank != 0:
        return
    line = {"metric": "compute_rdms seconds, FCI(10o,10e) ground state", "value": t_gpu, "unit": "s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_gpu * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic seeded integrals (seed %d)" % (1000 + nb),
            "config": {"workload": "compute_rdms of the FP64 ground state, FCI nbasis=10 5a5b (63504 dets)",
                       "ndet": int(ndet), "parallelism": "replicas"},
            "e2e": {"value": t_gpu, "unit": "s", "h2d_bytes_per_step": int(dets.nbytes + coeffs.nbytes),
                    "d2h_bytes_per_step": int(r1.nbytes + r2.nbytes)},
            "gpu_launches": launches, "clocks": clocks.summary()}
    if not args.skip_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        t0 = time.perf_counter()
        o1, o2 = O.compute_rdms(O.FULLCI, nb, na, nbeta, dets, coeffs)
        t_cpu = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": t_cpu, "unit": "s", "cores": 1, "kind": "port",
                                "sample": "the same call with the C oracle (serial restatement of pyci/src/rdm.cpp, "
                                          "which the reference runs on one thread)"}
        diff = max(float(np.abs(r1 - o1).max()), float(np.abs(r2 - o2).max()))
        line["parity"] = {"max_abs_diff_vs_oracle": diff, "ok": diff < 1e-12}
    print(json.dumps(line), flush=True)


def run_enpt2(args, world=1, rank=0, local=0):
    r"""compute_enpt2 on the 12-orbital 5a5b FCI Hamiltonian: the wave
    function is every determinant with |c| > 1e-4 in the full-space FP64
    ground state (colex order), solved in that subspace (FP64); the external
    space is the rest of the FCI space, eps = 1e-6.  value = seconds per call
    through the C ABI (host arrays in and out); the same call of the CPU oracle
    (serial restatement of pyci/src/enpt2.cpp, as the reference runs it with
    one thread) is the baseline, and the energies must agree to 1e-10 of the
    correction.  Replicas under torchrun."""
    import torch
    from math import comb
    import pyci_gb300 as pyci
    from pyci_gb300 import capi
    from pyci_gb300.synth import synthetic_integrals
    torch.cuda.set_device(local)
    nb, na, nbeta, eps = 12, 5, 5, 1.0e-6
    ctx = capi.Context(local)
    ecore, one, two = synthetic_integrals(nb, 1003)
    csr = capi.Csr(ctx, capi.WFN_FULLCI, nb, na, nbeta, None, one, two, flags=capi.BUILD_FULL_COLEX,
                   ndet=comb(nb, na) * comb(nb, nbeta))
    _, vecs, _ = csr.solve(n=1, tol=1e-8, ecore=ecore, mode=capi.SOLVE_FP64)
    csr.free()
    full = ctx.add_all_dets(capi.WFN_FULLCI, nb, na, nbeta)
    dets = np.ascontiguousarray(full[np.nonzero(np.abs(vecs[0]) > 1e-4)[0]])
    del full
    sub = capi.Csr(ctx, capi.WFN_FULLCI, nb, na, nbeta, dets, one, two)
    ev, cv, _ = sub.solve(n=1, tol=1e-10, ecore=ecore, mode=capi.SOLVE_FP64)
    sub.free()
    energy, coeffs = float(ev[0]), np.ascontiguousarray(cv[0])
    for _ in range(args.warmup):
        e2 = ctx.compute_enpt2(capi.WFN_FULLCI, nb, na, nbeta, dets, coeffs, one, two, energy, ecore, eps)
    lib = capi.lib()
    barrier(world)
    launches0 = lib.pyci_gpu_kernel_launches()
    times = []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e2 = ctx.compute_enpt2(capi.WFN_FULLCI, nb, na, nbeta, dets, coeffs, one, two, energy, ecore, eps)
            times.append(time.perf_counter() - t0)
    launches = (lib.pyci_gpu_kernel_launches() - launches0) // args.steps
    t_gpu = max_over_ranks(statistics.median(times), world)
    if rank != 0:
        return
    line = {"metric": "compute_enpt2 seconds, FCI(12o,10e) selected space", "value": t_gpu, "unit": "s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_gpu * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic seeded integrals (seed 1003)",
            "config": {"workload": "compute_enpt2 on FCI nbasis=12 5a5b: determinants with |c| > 1e-4 in the "
                                   "ground state, their subspace ground state, eps = 1e-6",
                       "ndet": int(dets.shape[0]), "energy": energy, "enpt2_energy": e2, "parallelism": "replicas"},
            "e2e": {"value": t_gpu, "unit": "s", "h2d_bytes_per_step": int(dets.nbytes + coeffs.nbytes + one.nbytes
                                                                           + two.nbytes),
                    "d2h_bytes_per_step": 8},
            "gpu_launches": launches, "clocks": clocks.summary()}
    if not args.skip_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        t0 = time.perf_counter()
        e_ref = O.compute_enpt2(O.FULLCI, nb, na, nbeta, dets, coeffs, one, two, energy, ecore, eps)
        t_cpu = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": t_cpu, "unit": "s", "cores": 1, "kind": "port",
                                "sample": "the same call with the C oracle (serial restatement of pyci/src/enpt2.cpp; "
                                          "the reference runs PYCI_NUM_THREADS = 1 threads by default)"}
        line["parity"] = {"oracle_energy": e_ref, "abs_diff": abs(e2 - e_ref),
                          "ok": abs(e2 - e_ref) <= 1e-10 * abs(e_ref - energy)}
    print(json.dumps(line), flush=True)


def run_profile_gram(args):
    r"""Profiling driver (for ncu): FP32 Gram products C = A^T B of --gram P Q N
    (random vectors, N rows), on the CUDA cores then on the tensor cores,
    --reps times each; prints the mean wall time per call of each."""
    import torch
    from pyci_gb300 import capi
    p, q, n = args.gram
    ctx = capi.Context(0)
    g = torch.Generator(device="cuda").manual_seed(0)
    a = torch.randn((p, n), device="cuda", generator=g)
    b = torch.randn((q, n), device="cuda", generator=g)
    out = {}
    for method, name in ((capi.GRAM_CUDA_CORES, "cuda_cores"), (capi.GRAM_TENSOR_CORES, "tensor_cores")):
        t0 = time.perf_counter()
        for _ in range(args.reps):
            ctx.gram_device(method, a.data_ptr(), p, b.data_ptr(), q, n)
        out[name + "_ms_per_call"] = (time.perf_counter() - t0) / args.reps * 1e3
    print(json.dumps({"profile": "gram", "p": p, "q": q, "n": n, **out}))


def run_profile_case(args):
    r"""Profiling driver (for ncu): build one FCI (or DOCI) operator and run
    its SpMM kernels (FP32 k=4, FP64 k=1, double-float k=4), or only mixed
    solves, with nothing else in the launch list."""
    import torch
    from pyci_gb300 import capi
    from pyci_gb300.synth import synthetic_integrals
    if args.profile == "gram":
        return run_profile_gram(args)
    nb, nu, nd = args.case
    ecore, one, two = synthetic_integrals(nb, 1000 + nb)
    from math import comb
    ctx = capi.Context(0)
    if args.wfn == "doci":
        csr = capi.Csr(ctx, capi.WFN_DOCI, nb, nu, nu, None, one, two, flags=capi.BUILD_FULL_COLEX,
                       ndet=comb(nb, nu))
    else:
        csr = capi.Csr(ctx, capi.WFN_FULLCI, nb, nu, nd, None, one, two, flags=capi.BUILD_FULL_COLEX,
                       ndet=comb(nb, nu) * comb(nb, nd))
    csr.prepare_mixed()
    N = csr.shape()[0]
    if args.profile == "spmm":
        x32 = torch.randn((N, 4), dtype=torch.float32, device="cuda")
        y32 = torch.empty_like(x32)
        x64 = torch.randn((N, 1), dtype=torch.float64, device="cuda")
        y64 = torch.empty_like(x64)
        xdf = torch.randn((N, 8), dtype=torch.float32, device="cuda")
        ydf = torch.empty((N, 4), dtype=torch.float64, device="cuda")
        # An operator whose CSR entries are deferred keeps them so: its FP64
        # product (which would write them) is left out.
        fp64 = not csr.storage() & capi.STORE_DEFERRED
        for _ in range(args.reps):
            csr.spmm_device(capi.PREC_FP32, 4, x32.data_ptr(), y32.data_ptr(), ctx.stream)
            if fp64:
                csr.spmm_device(capi.PREC_FP64, 1, x64.data_ptr(), y64.data_ptr(), ctx.stream)
            csr.spmm_device(capi.PREC_FP64_DF, 4, xdf.data_ptr(), ydf.data_ptr(), ctx.stream)
        torch.cuda.synchronize()
    else:
        for _ in range(args.reps):
            csr.solve(n=4, tol=TOL, ecore=ecore, mode=capi.SOLVE_MIXED)
    print(json.dumps({"profile": args.profile, "case": list(args.case), "ndet": N, "nnz_stored": csr.shape()[3]}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU baseline sample")
    ap.add_argument("--gram", type=int, nargs=3, default=[128, 8, 2 << 20], metavar=("P", "Q", "N"),
                    help="shape of --profile gram")
    ap.add_argument("--profile", choices=["spmm", "solve", "gram"], default=None,
                    help="profiling driver: only SpMM launches, or only mixed solves, on --case; "
                         "or only Gram products of shape --gram")
    ap.add_argument("--case", type=int, nargs=3, default=[11, 5, 5], metavar=("NBASIS", "NALPHA", "NBETA"))
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--wfn", choices=["fullci", "doci"], default="fullci", help="wave function of --case")
    ap.add_argument("--workload", choices=["fci12", "doci32", "fci8", "doci24", "batch64", "hci", "rdm", "enpt2"],
                    default="fci12",
                    help="fci12: the headline FCI(12o,10e) line; doci32: DOCI(32o, 8 pairs); fci8 / doci24: the "
                         "8-orbital FCI and 24-orbital DOCI cases; batch64: the 64-problem batched solve; "
                         "hci: one heat-bath CI selection step; rdm: compute_rdms of a FCI ground state; "
                         "enpt2: compute_enpt2 of a selected FCI space")
    args = ap.parse_args()
    global WORKLOAD, METRIC
    if args.workload in WORKLOADS:
        WORKLOAD = WORKLOADS[args.workload]
        METRIC = WORKLOAD["metric"]
    if args.profile:
        run_profile_case(args)
        return
    world, rank, local = dist_init(args)
    if args.workload in ("hci", "rdm", "enpt2"):
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference arm of this workload is the "
                                  "cpu_baseline of the ours line (the same call with the CPU oracle)"}), flush=True)
        elif args.workload == "hci":
            run_hci(args, world, rank, local)
        elif args.workload == "rdm":
            run_rdm(args, world, rank, local)
        else:
            run_enpt2(args, world, rank, local)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    if args.workload == "batch64":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched solver; "
                                  "its per-problem CPU path is timed by the default workload"}), flush=True)
        else:
            run_batch(args, world, rank, local)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
