"""Benchmark: GPU cell assembly (scikit-fem's BilinearForm.assemble) on GB300.

Default workload: TetP1 k*dot(grad u, grad v) + u*v on the unit-cube tensor
mesh with 101 nodes per axis (6,000,000 tets, 1,030,301 nodes), per-element
k ~ lognormal(0, 1) (seeded), float64, plain forward assembly to CSR.

One step = one plain assembly of the whole mesh into its CSR pattern, inputs
resident in HBM: the coefficient checks, then the one-pass P1 assembly --
each CSR row contracts the form per (cell, local row) from the basis's
per-cell geometry cache (what CellBasis keeps of its mapping) and sums the
contributions in a fixed order.  Nothing of an earlier call is reused: the
form is contracted and summed every step.  The working set (geometry 528 MB,
incidence and slots 290 MB, CSR 122 MB) is far larger than L2, so no flush
is needed between steps.  ``e2e`` times the public API call a user makes --
``form.assemble(basis, k=<(nelems, nqp) host array>)`` returning a
scipy.sparse.csr_matrix -- including the host->device copy of k and the
device->host copy of the CSR.

``--impl reference`` times the CPU oracle (the numpy restatement of
scikit-fem's assembly, its local loop split over all host threads as
BilinearForm(nthreads=...) does) on the same 101^3 workload: each step is
``assemble`` on a prebuilt basis, like the GPU step; one Basis + assemble
run is reported beside it, as scikit-fem's performance.py times it.
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, os.path.join(ROOT, "scikit-fem_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "elements/s & %HBM roofline: plain vs adjoint/batched assemble, rel err <=1e-12"
UNIT = "elements/s"

# DRAM bytes per cell of the kernels, from ncu captures of one launch each
# on the 61^3-node cube (1,296,000 cells) -- the one-pass sum and the
# coefficient checks of the step; the two-pass kernels (local kernel on the
# cached geometry, staging sum) and the opt-in coefficient-update sum for
# comparison.  The one-pass sum's figure is per form (fem_set_onepass
# variant: 0 row form, 1 upper-gather form, 2 upper form with TMA-staged codes);
# the upper-gather form's is from one launch at the full 101^3 size (6M cells,
# upper entries in blocks of 4,096 rows: 1.06 GB read + 147.7 MB written).
ONEPASS_B_PER_CELL = {0: 159.7, 1: 185.6, 2: 185.6}
ONEPASS_B_SOURCE = {0: "one launch at 1.3M cells", 1: "one launch at 6M cells (this workload)",
                    2: "one launch at 1.3M cells"}
ONEPASS_KERNEL = {0: "csr_geometry_p1_kernel<4,U,0> (one-pass P1 sum, row form)",
                  1: "csr_upper_p1_kernel<4,U,0> (one-pass P1 sum, upper-gather form)",
                  2: "csr_upper_p1_tma_kernel<4,U,0> (one-pass P1 sum, TMA-staged codes)"}
CHECK_B_PER_CELL = 9.0
FOLDED_CHECK_B_PER_CELL = 1.0   # the zero-bit byte, read inside the one-pass sum
LOCAL_B_PER_CELL = 233.0
SUM_B_PER_CELL = 193.9
FUSED_B_PER_CELL = 218.5
# FP64 operations per cell of the one-pass vector TetP2 elasticity: the pair
# blocks (geometry ~70, E ~250) and the node blocks' reference-tensor terms
# (1,194 FMAs for the 55 blocks on and above the block diagonal)
VEC_TETP2_FP64_PER_CELL = 70 + 250 + 1194
# FP64 operations per cell of the one-pass scalar TetP2 k*Laplace + mass: the
# pair values (10 products of k and the cached Gram entries, 2 for the mass
# scale) and the CSR entries' reference-tensor terms (136 FMAs for the 55
# node pairs on and above the diagonal, symmetric terms merged) and mass (55)
SCALAR_TETP2_FP64_PER_CELL = 12 + 136 + 55
TRAFFIC_SOURCE = "ncu dram__bytes_read+write of one launch on the 1.3M-cell case, per cell"


def max_over_ranks(ms, dist=None, device="cpu"):
    """Replicas: every rank times its own copy of the workload; the job's
    step time is the slowest rank's (one all-reduce, after the timed region)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(cells_per_rank, world, ms):
    """Whole-job throughput of ``world`` replicas: all cells of all ranks
    over the slowest rank's step time."""
    return cells_per_rank * world / (ms * 1e-3)


def algorithmic_bytes(nelems, nverts, nnz, dim=3, nloc=4):
    return nelems * (nloc * 4 + 8) + nverts * dim * 8 + nnz * 8


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# measured DFMA throughput of this GB300 pool (fp64_probe: 0.598e12 FMA/s)
FP64_PEAK_GFLOPS = 1195.0


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ workloads
# Seeded synthetic inputs of the benchmark configurations (the tests build
# the same ones to check them against the oracle at these sizes).

SEED = 20261203


def build_workload(n_nodes, seed=SEED):
    """TetP1 k*Laplace + mass: MeshTet.init_tensor with n_nodes per axis
    (6 tets per cube), per-cell k ~ lognormal(0, 1)."""
    import skfem_gb300 as F
    m = F.MeshTet.init_tensor(*(np.linspace(0, 1, n_nodes),) * 3)
    rng = np.random.default_rng(seed)
    k = rng.lognormal(0.0, 1.0, m.nelements)
    return m, k


def tri_square(n_cells=256):
    """TriP1 Laplace + unit load: the unit square as n x n squares, each cut
    into two triangles."""
    import skfem_gb300 as F
    x = np.linspace(0, 1, n_cells + 1)
    return F.MeshTri.init_tensor(x, x)


def jittered_tet_cube(n_cells, seed=SEED + 3):
    """Vector TetP2 elasticity mesh: n^3 cubes x 6 tets, interior nodes
    moved uniformly by up to 0.2 h per axis."""
    import skfem_gb300 as F
    m = F.MeshTet.init_tensor(*(np.linspace(0, 1, n_cells + 1),) * 3)
    p = m.p.copy()
    inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
    rng = np.random.default_rng(seed)
    p[:, inner] += rng.uniform(-0.2 / n_cells, 0.2 / n_cells, size=(3, int(inner.sum())))
    return F.MeshTet(p, m.t)


def hex_cube_workload(n_cells, seed=SEED + 4, jitter=0.0):
    """Hex1 theta*Laplace: n^3 hexahedra (interior nodes jittered by up to
    jitter * h per axis when jitter > 0: isoparametric cells), theta ~
    U[0.01, 1] per cell, adjoint vectors w, u ~ N(0, 1)."""
    import skfem_gb300 as F
    m = F.MeshHex.init_tensor(*(np.linspace(0, 1, n_cells + 1),) * 3)
    rng = np.random.default_rng(seed)
    if jitter > 0:
        p = m.p.copy()
        inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
        p[:, inner] += rng.uniform(-jitter / n_cells, jitter / n_cells,
                                   size=(3, int(inner.sum())))
        m = F.MeshHex(p, m.t)
    theta = rng.uniform(0.01, 1.0, m.nelements)
    w = rng.standard_normal(m.p.shape[1])
    u = rng.standard_normal(m.p.shape[1])
    return m, theta, w, u


def trip2_batch(n_meshes, seed=SEED + 5):
    """Batched TriP2 k*Laplace: meshes of log-uniform cell counts in
    [2k, 200k], each a jittered unit-square grid, k ~ lognormal(0, 0.5)."""
    import skfem_gb300 as F
    rng = np.random.default_rng(seed)
    cells = np.exp(rng.uniform(np.log(2e3), np.log(2e5), n_meshes))
    meshes, ks = [], []
    for c in cells:
        nn = max(1, int(round(np.sqrt(c / 2))))
        mm = F.MeshTri.init_tensor(np.linspace(0, 1, nn + 1), np.linspace(0, 1, nn + 1))
        pp = mm.p.copy()
        inner = np.all((pp > 1e-12) & (pp < 1 - 1e-12), axis=0)
        pp[:, inner] += rng.uniform(-0.2 / nn, 0.2 / nn, size=(2, int(inner.sum())))
        meshes.append(F.MeshTri(pp, mm.t))
        ks.append(rng.lognormal(0.0, 0.5, mm.nelements))
    return meshes, ks


def k_laplace_mass_form():
    import skfem_gb300 as F
    from skfem_gb300 import helpers as H

    @F.BilinearForm
    def form(u, v, w):
        return w.k * H.dot(H.grad(u), H.grad(v)) + u * v
    return form


def gpu_arm(args):
    import torch

    import skfem_gb300 as F
    from skfem_gb300 import _native as N

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    m, k = build_workload(args.nodes, SEED + rank)
    b = F.Basis(m, F.ElementTetP1())
    form = k_laplace_mass_form()

    kd = torch.from_numpy(k).cuda()
    # first call builds the pattern and the per-cell geometry cache (one-time,
    # reported separately: the basis's setup, as CellBasis.__init__ is)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    K0 = form.assemble_torch(b, k=kd)
    torch.cuda.synchronize()
    pattern_s = time.perf_counter() - t0
    entry = next(iter(b._patterns.values()))
    nnz = entry.nnz
    nel = m.nelements
    # launch parameters by the autotuner on this workload (setup, untimed)
    from skfem_gb300 import autotune
    tuned, timings = autotune.tune(form, b, {"k": kd}, reps=3, use_cache=False)
    # the fastest configuration of each form of the one-pass sum (0 two lanes
    # per row, 1 a lane per upper entry, 2 the same with TMA-staged codes)
    variant_ms = {}
    for t_ms, cfg in timings:
        v = str(cfg.get("onepass", 1))
        variant_ms[v] = min(variant_ms.get(v, float("inf")), t_ms)
    if args.onepass is not None:
        tuned = dict(tuned, onepass=args.onepass)
        autotune.apply(N.FAMILY["TetP1"], tuned)

    # a bare C-ABI step: inputs in HBM, results in HBM
    coeffs, ch, c_form = form._setup(b, None, {"k": kd})
    vals = torch.empty(nnz, dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib = N.lib()
    stream = torch.cuda.current_stream()
    sp = N.stream_ptr(stream)

    def step():
        N.check(lib.fem_assemble(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                                 entry.pat.handle, N.ptr(entry.staging), N.ptr(vals),
                                 N.ptr(status), sp))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        time.sleep(0.3)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
        time.sleep(0.2)
    ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps, dist, "cuda")
    assert int(status.item()) == 0, "assembly status %d" % int(status.item())
    assert torch.equal(vals, K0.values()), "repeated assembly not bitwise identical"

    # per-kernel split (same stream, CUDA events): the step is the
    # coefficient checks and the one-pass sum; the same call without a
    # status runs the one-pass sum alone.  For comparison, the two-pass
    # kernels (the local kernel on the cached geometry + the staging sum, as
    # fem_assemble_local and fem_csr_sum_staged run them) and the local
    # kernel computing its geometry from the coordinates
    local_buf = entry.staging
    # the two-pass kernels at their own default launch shape (the tuned one
    # is chosen for the one-pass sum and does not apply to them)
    autotune.apply(N.FAMILY["TetP1"], dict(tuned, local_block=128, persistent=0))
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    t_local, t_sum, t_geom, t_one = 0.0, 0.0, 0.0, 0.0
    reps = max(3, args.steps)
    two_pass = torch.empty_like(vals)
    for _ in range(reps):
        e0.record(stream)
        N.check(lib.fem_assemble(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                                 entry.pat.handle, N.ptr(entry.staging), N.ptr(vals), None, sp))
        e1.record(stream)
        torch.cuda.synchronize()
        t_one += e0.elapsed_time(e1)
        e0.record(stream)
        N.check(lib.fem_assemble_local(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                                       entry.pat.handle, N.ptr(local_buf), N.ptr(status), 0, nel,
                                       sp))
        e1.record(stream)
        N.check(lib.fem_csr_sum_staged(entry.pat.handle, N.ptr(local_buf), N.ptr(two_pass), sp))
        e2.record(stream)
        torch.cuda.synchronize()
        t_local += e0.elapsed_time(e1)
        t_sum += e1.elapsed_time(e2)
        e0.record(stream)
        N.check(lib.fem_local_matrices(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                                       N.ptr(local_buf), sp))
        e1.record(stream)
        torch.cuda.synchronize()
        t_geom += e0.elapsed_time(e1)
    # the local kernel with each tile's geometry staged by a 2-D TMA tensor
    # copy (fem_set_local_tma), against its coalesced loads above
    N.check(lib.fem_assemble_local(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                                   entry.pat.handle, N.ptr(local_buf), N.ptr(status), 0, nel, sp))
    torch.cuda.synchronize()
    local_ref = local_buf.clone()
    t_local_tma = 0.0
    lib.fem_set_local_tma(N.FAMILY["TetP1"], 1)
    try:
        for _ in range(reps + 1):
            e0.record(stream)
            N.check(lib.fem_assemble_local(N.byref(b.c_mesh), N.byref(b.c_basis),
                                           N.byref(c_form), entry.pat.handle, N.ptr(local_buf),
                                           N.ptr(status), 0, nel, sp))
            e1.record(stream)
            torch.cuda.synchronize()
            t_local_tma += e0.elapsed_time(e1) if _ else 0.0   # the first is a warm-up
    finally:
        lib.fem_set_local_tma(N.FAMILY["TetP1"], 0)
    assert int(status.item()) == 0, "TMA-staged local kernel status %d" % int(status.item())
    local_tma_same = bool(torch.equal(local_buf, local_ref))
    t_local_tma /= reps
    autotune.apply(N.FAMILY["TetP1"], tuned)
    t_local /= reps
    t_sum /= reps
    t_geom /= reps
    t_one /= reps
    t_checks = max(0.0, ms - t_one)
    d = (two_pass - vals).abs().max().item() / vals.abs().max().item()

    # the opt-in coefficient-update cache (cached unit-coefficient stiffness
    # rows and mass matrix; a form re-assembled with new k many times): one
    # fused sum per call -- reported beside the plain step, not as it
    form.cache_coefficient_update(b, k=kd)
    t_cu = _time(step, reps)
    lib.fem_pattern_drop_coefficient_update(entry.pat.handle)
    entry.coef_update = False
    b.__dict__.pop("_coef_update", None)
    step()
    torch.cuda.synchronize()
    assert torch.equal(vals, K0.values())

    # e2e: public API with host buffers (k as the reference takes it)
    kw_host = b.zero_w() + k[:, None]
    for _ in range(3):
        form.assemble(b, k=kw_host)
    torch.cuda.synchronize()
    e2e_steps = max(5, args.steps)
    e2e_times = []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        Kh = form.assemble(b, k=kw_host)
        e2e_times.append(time.perf_counter() - t0)
        del Kh
    Kh = form.assemble(b, k=kw_host)
    assert np.array_equal(Kh.data, K0.values().cpu().numpy()), "e2e values differ from the step"
    e2e_s = sum(e2e_times) / len(e2e_times)
    h2d = kw_host.nbytes
    d2h = Kh.data.nbytes + Kh.indices.nbytes + Kh.indptr.nbytes

    hbm, peak_kind = peaks()
    Bytes = algorithmic_bytes(nel, m.p.shape[1], nnz)
    achieved = Bytes / (ms * 1e-3) / 1e9
    # FP64 work of the TetP1 local kernel computing its geometry, per cell,
    # from its ncu instruction counts: 18 DADD + 21 DMUL + 38 DFMA (2 FLOP each)
    flops_per_el = 115.0
    fp64_achieved = nel * flops_per_el / (t_geom * 1e-3) / 1e9

    def kern(name, t, bpc):
        out = {"kernel": name, "ms": t, "dram_bytes_per_cell": bpc}
        if bpc is not None and t > 0:
            out["gbs"] = bpc * nel / (t * 1e-3) / 1e9
            out["frac_hbm"] = out["gbs"] / hbm
        return out

    one_form = int(tuned.get("onepass", 1))
    one_bpc = ONEPASS_B_PER_CELL.get(one_form)
    # the plain upper form checks the coefficients itself (one byte of the
    # pattern's zero bits per cell); the other forms run the checks kernel
    folded = one_form == 1
    check_bpc = FOLDED_CHECK_B_PER_CELL if folded else CHECK_B_PER_CELL
    traffic = None if one_bpc is None else (one_bpc + check_bpc) * nel
    res = {
        "metric": METRIC, "value": replica_value(nel, world, ms), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak" if world > 1 else "replicas only",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded tensor mesh, lognormal k)",
        "config": {"workload": "TetP1 k*laplace+mass, 101^3-node unit cube tensor mesh, 6 tets/cell",
                   "nelems": nel, "nverts": int(m.p.shape[1]), "nnz": nnz,
                   "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas",
                   "pattern_build_s": pattern_s, "autotuned": tuned,
                   "step": "plain assembly: one-pass sum contracting the form per cell row "
                           "from the per-cell geometry cache (Gram matrix of the barycentric "
                           "gradients / (6|det|), |det|) -- the mapping data CellBasis keeps; "
                           "the form is contracted and summed every step -- with the "
                           "coefficient checks (folded into the sum in its plain upper form, "
                           "a separate kernel otherwise)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic,
                     "traffic_source": (None if traffic is None else
                                        "ncu dram__bytes_read+write, %s: one-pass sum %.1f + "
                                        "checks %.1f B/cell" % (ONEPASS_B_SOURCE[one_form],
                                                                one_bpc, check_bpc)),
                     "peak_kind": peak_kind, "algorithmic_bytes_per_step": Bytes,
                     "kernel": "whole assembly step (coefficient checks + one-pass sum)",
                     "fp64_floor_ms": nel * 16 / 0.598e12 * 1e3},
        "kernels": {
            "onepass_sum": kern(ONEPASS_KERNEL[one_form], t_one, one_bpc),
            "coef_checks": kern(("folded into the one-pass sum (its zero-bit compare at each "
                                 "cell's diagonal contribution; step time minus the sum alone)")
                                if folded else
                                "coef_fields_kernel (step time minus the one-pass sum)",
                                t_checks, check_bpc),
            "two_pass_local": kern("simplex_scalar_kernel<3,1,BS,cached geometry>", t_local,
                                   LOCAL_B_PER_CELL),
            "two_pass_sum": kern("csr_sum_kernel<4,U,0>", t_sum, SUM_B_PER_CELL),
            "two_pass_local_tma": dict(kern("simplex_scalar_kernel<3,1,128,cached,TMA> (each tile's "
                                            "geometry by one cp.async.bulk.tensor.2d copy)",
                                            t_local_tma, LOCAL_B_PER_CELL),
                                       bitwise_equal=local_tma_same),
            "coefficient_update_sum": kern("csr_scaled_pair_kernel<4,U> (opt-in cache of "
                                           "unit-coefficient rows and mass matrix; not the "
                                           "plain step)", t_cu, FUSED_B_PER_CELL),
            "bytes_source": TRAFFIC_SOURCE,
            "two_pass_vs_onepass_max_rel": d,
            "onepass_variants_best_ms": variant_ms},
        "fp64": {"kernel": "local matrices computing their geometry (fem_local_matrices; the "
                           "step reads the basis's cached geometry instead)",
                 "ms": t_geom, "gflops": fp64_achieved, "peak_gflops": FP64_PEAK_GFLOPS,
                 "frac": fp64_achieved / FP64_PEAK_GFLOPS},
        "kernels_ms": {"onepass_sum": t_one, "coef_checks": t_checks,
                       "two_pass_local": t_local, "two_pass_local_tma": t_local_tma,
                       "two_pass_sum": t_sum,
                       "two_pass_step": t_local + t_sum,
                       "coefficient_update_step": t_cu,
                       "local_computing_geometry": t_geom},
        "clocks": clk.summary(),
        "e2e": {"value": nel / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "s_per_step": e2e_s,
                "s_per_step_median": sorted(e2e_times)[len(e2e_times) // 2],
                "api": "BilinearForm.assemble(basis, k=(nelems, nqp) host array) -> scipy CSR"},
        # per step: the one-pass sum (+ the checks kernel unless folded)
        "gpu_launches": (1 if folded else 2) * args.steps,
    }
    if rank == 0 and not args.no_cpu:
        res["cpu_baseline"], res["parity"] = cpu_baseline(args)
    if rank == 0 and not args.no_secondary:
        res["secondary"] = secondary_workloads(args)
    if dist:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(res))


def _time(fn, reps, warm=2):
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _cpu_oracle(assemble, cells, sample):
    """The oracle (the numpy restatement of the reference) on a bounded
    sample of a workload, on all host threads: cells per second of one run."""
    t0 = time.perf_counter()
    assemble()
    s = time.perf_counter() - t0
    return {"cells_per_s": cells / s, "s": s, "cores": os.cpu_count() or 1, "kind": "port",
            "sample": sample}


def _abi_step(F, N, form, b, coefs):
    """Bare C-ABI assembly step (inputs and outputs in HBM)."""
    import torch
    form.assemble_torch(b, **coefs)
    entry = next(e for k, e in b._patterns.items() if k[0] == "bilinear")
    _, _, c_form = form._setup(b, None, coefs)
    vals = torch.empty(entry.nnz, dtype=torch.float64, device="cuda")
    lib = N.lib()

    def step():
        N.check(lib.fem_assemble(N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form),
                                 entry.pat.handle, N.ptr(entry.staging), N.ptr(vals), None,
                                 N.stream_ptr()))
    return step, entry, c_form, vals


def secondary_workloads(args, only=None):
    """The other workloads of the assembly path, each timed on the device.
    ``only`` restricts the run to one of tri_p1 / tet_p2 / tet_p2_vec /
    hex1_vjp / batched / generic / condense (sizes from --p2-n, --vec-n,
    --hex-n, --batch, --generic-n, --nodes)."""
    want = (lambda name: only is None or only == name)
    import torch

    import skfem_gb300 as F
    from skfem_gb300 import _native as N
    from skfem_gb300 import helpers as H
    from skfem_gb300.models.elasticity import linear_elasticity
    from skfem_gb300.models.poisson import laplace, unit_load
    from skfem_gb300.form import _Coefficients

    hbm, _ = peaks()
    out = {}
    rng = np.random.default_rng(args.seed)
    # the oracle on a bounded sample of each workload, all host threads
    cpu = not getattr(args, "no_cpu", False)
    nthr = os.cpu_count() or 1
    if cpu:
        import oracle as O
    reps = 10
    lib = N.lib()

    if want('tri_p1'):
        # cfg1: TriP1 Laplace + unit load, 256x256 squares (131,072 triangles)
        m = F.MeshTri.init_tensor(np.linspace(0, 1, 257), np.linspace(0, 1, 257))
        b = F.Basis(m, F.ElementTriP1())
        step, entry, _, _ = _abi_step(F, N, laplace, b, {})
        ms_k = _time(step, reps)
        ms_b = _time(lambda: unit_load.assemble_torch(b), reps)
        B = m.nelements * (3 * 4) + m.p.size * 8 + entry.nnz * 8
        out["tri_p1_laplace_256"] = {
            "nelems": m.nelements, "nnz": entry.nnz, "ms_matrix": ms_k, "ms_load": ms_b,
            "elements_per_s": m.nelements / ((ms_k + ms_b) * 1e-3),
            "hbm_frac_matrix": B / (ms_k * 1e-3) / 1e9 / hbm}
        if cpu:
            om = O.mesh_tri_tensor(np.linspace(0, 1, 257), np.linspace(0, 1, 257))
            ob = O.OBasis(om, O.TriP1())
            c = _cpu_oracle(lambda: (O.bilinear_assemble(O.laplace, ob, nthreads=nthr),
                                     O.linear_assemble(O.unit_load, ob)),
                            om.nelements, "the whole workload (matrix + load), prebuilt basis")
            out["tri_p1_laplace_256"]["cpu_oracle"] = c
            out["tri_p1_laplace_256"]["speedup_vs_cpu_oracle"] = (
                out["tri_p1_laplace_256"]["elements_per_s"] / c["cells_per_s"])

    if want('tet_p2_vec'):
        # cfg3: vector TetP2 elasticity, 41^3 nodes jittered +-0.2h, lambda=1, mu=0.5
        n = args.vec_n
        m = jittered_tet_cube(n)
        b = F.Basis(m, F.ElementVector(F.ElementTetP2()), intorder=4)
        form = linear_elasticity(1.0, 0.5)
        t0 = time.perf_counter()
        step, entry, c_form, vals = _abi_step(F, N, form, b, {})
        torch.cuda.synchronize()
        build_s = time.perf_counter() - t0
        ms = _time(step, 5)
        first = vals.clone()
        step()
        torch.cuda.synchronize()
        same = bool(torch.equal(first, vals))
        lib = N.lib()
        # the two-pass path for comparison: local matrices into the staging
        # (block-upper layout), then the fixed-order segmented sum
        fam = N.FAMILY["TetP2"]
        try:
            # the one-pass sum's cooperative form (the D*D lanes of a node block
            # together), bitwise the same values
            lib.fem_set_onepass(fam, 2)
            ms_coop = _time(step, 5)
            coop_same = bool(torch.equal(first, vals))
            lib.fem_set_onepass(fam, 0)
            ms_two = _time(step, 3)
            dev = float(((vals - first).abs().max() / first.abs().max()).item())
            ms_local = _time(lambda: N.check(lib.fem_assemble_local(
                N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form), entry.pat.handle,
                N.ptr(entry.staging), None, 0, b.nelems, N.stream_ptr())), 3)
        finally:
            lib.fem_set_onepass(fam, 1)
        B = m.nelements * (10 * 4) + m.p.size * 8 + entry.nnz * 8
        out["tet_p2_vec_elasticity_%d" % (n + 1)] = {
            "nelems": m.nelements, "ndofs": b.N, "nnz": entry.nnz, "ms": ms,
            "step": "one-pass vector sum: the cells' pair blocks, then one lane per node block "
                    "contracting the reference tensor while it sums (no local matrices stored)",
            "repeat_bitwise_equal": same,
            "ms_onepass_coop": ms_coop, "coop_bitwise_equal": coop_same,
            "ms_two_pass": ms_two, "ms_two_pass_local": ms_local,
            "two_pass_vs_onepass_max_rel": dev,
            "pattern_build_s": build_s, "elements_per_s": m.nelements / (ms * 1e-3),
            "hbm_frac": B / (ms * 1e-3) / 1e9 / hbm, "algorithmic_bytes": B,
            "fp64_floor_ms": m.nelements * VEC_TETP2_FP64_PER_CELL / 0.598e12 * 1e3}
        if cpu:
            sm = jittered_tet_cube(16)
            ob = O.OBasis(O.OMesh(np.asarray(sm.p), np.asarray(sm.t), "tet"),
                          O.Vector(O.TetP2()), intorder=4)
            c = _cpu_oracle(lambda: O.bilinear_assemble(O.linear_elasticity(1.0, 0.5), ob,
                                                        nthreads=nthr),
                            sm.nelements, "16^3 cubes jittered the same way (%d tets), prebuilt "
                                          "basis" % sm.nelements)
            key = "tet_p2_vec_elasticity_%d" % (n + 1)
            out[key]["cpu_oracle"] = c
            out[key]["speedup_vs_cpu_oracle"] = out[key]["elements_per_s"] / c["cells_per_s"]
        del step, entry, vals, b
        torch.cuda.empty_cache()

    if want('tet_p2'):
        # plain scalar TetP2 k*Laplace + mass (the TetP1 workload's form and
        # lognormal k at second order) on the 61^3-node cube, 1,296,000 cells
        m, k = build_workload(args.p2_n)
        b = F.Basis(m, F.ElementTetP2())
        kd = torch.tensor(k, device="cuda")

        @F.BilinearForm
        def k_laplace_mass(u, v, w):
            return w.k * H.dot(H.grad(u), H.grad(v)) + u * v

        t0 = time.perf_counter()
        step, entry, c_form, vals = _abi_step(F, N, k_laplace_mass, b, {"k": kd})
        torch.cuda.synchronize()
        build_s = time.perf_counter() - t0
        fam = N.FAMILY["TetP2"]
        from skfem_gb300 import autotune
        try:
            # launch shape and the one-pass sum's form (per contribution / one
            # FMA per step: the same bits) by the autotuner
            tuned, _ = autotune.tune(k_laplace_mass, b, {"k": kd}, reps=3, use_cache=False)
            ms = _time(step, 5)
            first = vals.clone()
            step()
            torch.cuda.synchronize()
            same = bool(torch.equal(first, vals))
            form_ms = {}
            for v in (1, 2):
                lib.fem_set_onepass(fam, v)
                form_ms[v] = _time(step, 5)
                same = same and bool(torch.equal(first, vals))
            # the two-pass path: local matrices into the staging, then the
            # fixed-order segmented sum
            lib.fem_set_onepass(fam, 0)
            ms_two = _time(step, 3)
            dev = float(((vals - first).abs().max() / first.abs().max()).item())
            ms_local = _time(lambda: N.check(lib.fem_assemble_local(
                N.byref(b.c_mesh), N.byref(b.c_basis), N.byref(c_form), entry.pat.handle,
                N.ptr(entry.staging), None, 0, b.nelems, N.stream_ptr())), 3)
        finally:
            # the library's default tuning for the later workloads of the family
            autotune.apply(fam, {"local_block": 128, "persistent": 0, "sum_unroll": 8,
                                 "sum_cols": 1, "onepass": 1})
        B = m.nelements * (10 * 4 + 8) + m.p.size * 8 + entry.nnz * 8
        out["tet_p2_k_laplace_mass_%d" % args.p2_n] = {
            "nelems": m.nelements, "ndofs": b.N, "nnz": entry.nnz, "ms": ms,
            "step": "one-pass node-block sum: per cell the 10 scaled Gram entries times k and "
                    "the mass scale, then one lane per CSR entry on and above the diagonal "
                    "contracting the reference tensor while it sums (no local matrices stored)",
            "autotuned": tuned,
            "forms_and_repeats_bitwise_equal": same,
            "ms_onepass_per_contribution": form_ms[1], "ms_onepass_flat": form_ms[2],
            "ms_two_pass": ms_two, "ms_two_pass_local": ms_local,
            "two_pass_vs_onepass_max_rel": dev,
            "pattern_build_s": build_s, "elements_per_s": m.nelements / (ms * 1e-3),
            "hbm_frac": B / (ms * 1e-3) / 1e9 / hbm, "algorithmic_bytes": B,
            "fp64_floor_ms": m.nelements * SCALAR_TETP2_FP64_PER_CELL / 0.598e12 * 1e3}
        if cpu:
            om = O.mesh_tet_tensor(*(np.linspace(0, 1, 41),) * 3)
            kc = np.random.default_rng(SEED).lognormal(0.0, 1.0, om.nelements)
            ob = O.OBasis(om, O.TetP2())
            c = _cpu_oracle(lambda: O.bilinear_assemble(O.k_laplace_mass, ob,
                                                        k=ob.zero_w() + kc[:, None],
                                                        nthreads=nthr),
                            om.nelements, "the 41^3-node cube (%d tets), prebuilt basis"
                                          % om.nelements)
            key = "tet_p2_k_laplace_mass_%d" % args.p2_n
            out[key]["cpu_oracle"] = c
            out[key]["speedup_vs_cpu_oracle"] = out[key]["elements_per_s"] / c["cells_per_s"]
        del step, entry, vals, b
        torch.cuda.empty_cache()

    if want('hex1_vjp'):
        # cfg4: Hex1 theta*Laplace 64^3 cells: plain assembly vs forward + adjoint,
        # on the tensor cube (parallelepiped cells: closed form) and on the same
        # cube with interior nodes jittered by up to 0.2 h (isoparametric
        # cells: the 4x4x4-point quadrature and its adjoint)
        from skfem_gb300.autodiff import _vertex_incidence

        @F.BilinearForm
        def theta_laplace(u, v, w):
            return w.theta * H.dot(H.grad(u), H.grad(v))

        for jit in args.hex_jitter:
            tag = "_jittered" if jit > 0 else ""
            m, theta_h, w_h, u_h = hex_cube_workload(args.hex_n, jitter=jit)
            b = F.Basis(m, F.ElementHex1())
            theta = torch.tensor(theta_h, device="cuda")
            w = torch.tensor(w_h, device="cuda")
            u = torch.tensor(u_h, device="cuda")
            step, entry, c_form, vals = _abi_step(F, N, theta_laplace, b, {"theta": theta})
            vinc = _vertex_incidence(b)
            dth = torch.empty(m.nelements, dtype=torch.float64, device="cuda")
            dX = torch.empty_like(b.p_dev)
            scratch = torch.empty(m.nelements * 24, dtype=torch.float64, device="cuda")

            def vjp():
                N.check(lib.fem_bilinear_vjp(N.byref(b.c_mesh), N.byref(b.c_basis),
                                             N.byref(c_form), vinc.handle, N.ptr(w), N.ptr(u),
                                             N.ptr(dth), None, N.ptr(dX), N.ptr(scratch),
                                             N.stream_ptr()))

            ms_f = _time(step, reps)
            ms_v = _time(vjp, reps)
            ms_fv = _time(lambda: (step(), vjp()), reps)
            out["hex1_theta_laplace_%d%s_vjp" % (args.hex_n, tag)] = {
                "nelems": m.nelements, "nnz": entry.nnz, "ms_forward": ms_f, "ms_vjp": ms_v,
                "ms_forward_plus_vjp": ms_fv, "vjp_over_forward": ms_fv / ms_f,
                "elements_per_s_forward": m.nelements / (ms_f * 1e-3),
                "cells": "isoparametric (64-point quadrature)" if jit else
                         "parallelepipeds (closed form)"}
            if cpu:
                sm, th_s, _, _ = hex_cube_workload(args.hex_n, jitter=jit)
                ob = O.OBasis(O.OMesh(np.asarray(sm.p), np.asarray(sm.t), "hex"), O.Hex1())
                c = _cpu_oracle(lambda: O.bilinear_assemble(O.theta_laplace, ob,
                                                            theta=ob.zero_w() + th_s[:, None],
                                                            nthreads=nthr),
                                sm.nelements, "the whole workload, forward assembly, "
                                              "prebuilt basis")
                key = "hex1_theta_laplace_%d%s_vjp" % (args.hex_n, tag)
                out[key]["cpu_oracle"] = c
                out[key]["speedup_vs_cpu_oracle"] = (out[key]["elements_per_s_forward"] /
                                                     c["cells_per_s"])
            del step, entry, vals, b, scratch
            torch.cuda.empty_cache()

    if want('batched'):
        # cfg5: 512 jittered TriP2 squares, cells log-uniform in [2k, 200k], forward + adjoint
        from skfem_gb300.batched import BatchedBasis, GraphedAssembly
        meshes, ks = trip2_batch(args.batch)
        brng = np.random.default_rng(SEED + 6)

        @F.BilinearForm
        def k_laplace(u, v, w):
            return w.k * H.dot(H.grad(u), H.grad(v))

        t0 = time.perf_counter()
        bb = BatchedBasis(meshes, F.ElementTriP2())
        kk = torch.tensor(np.concatenate(ks), device="cuda")
        wb = torch.tensor(brng.standard_normal(bb.N), device="cuda")
        ub = torch.tensor(brng.standard_normal(bb.N), device="cuda")
        from skfem_gb300 import autotune
        best, _ = autotune.tune(k_laplace, bb, {"k": kk}, reps=2, use_cache=False)
        # one persistent work-queue launch per step (forward + coefficient adjoint)
        ga = GraphedAssembly(k_laplace, bb, {"k": kk}, w=wb, u=ub).capture()
        torch.cuda.synchronize()
        setup_s = time.perf_counter() - t0
        ms_graph = _time(ga.replay, 5)
        ga.check()
        # the same union with the separate kernels (local, staging sum, adjoint)
        gs = GraphedAssembly(k_laplace, bb, {"k": kk}, w=wb, u=ub, persistent=False).capture()
        ms_union = _time(gs.replay, 5)
        gs.check()
        # per-mesh plain launches of the same work (fem_assemble + the adjoint
        # kernel per mesh, patterns and geometry prebuilt): eager, and all of
        # them captured into one CUDA graph (no host launch cost, only the
        # kernels and the gaps between them)
        per = []
        for mm, kv in zip(meshes, ks):
            bm = F.Basis(mm, F.ElementTriP2())
            kt = torch.tensor(kv, device="cuda")
            g1 = GraphedAssembly(k_laplace, bm, {"k": kt},
                                 w=torch.zeros(bm.N, dtype=torch.float64, device="cuda"),
                                 u=torch.zeros(bm.N, dtype=torch.float64, device="cuda"),
                                 persistent=False)
            per.append(g1)
        ms_loop = _time(lambda: [g.run_eager() for g in per], 3, warm=1)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for g in per:
                g.run_eager()
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        loop_graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(loop_graph):
            for g in per:
                g.run_eager()
        ms_loop_graph = _time(loop_graph.replay, 3, warm=1)
        # per-mesh calls through the public API (assemble + autograd adjoint), as a
        # user without the batched path would write them
        from skfem_gb300.autodiff import assemble_vjp
        api = []
        for mm, kv, g1 in zip(meshes, ks, per):
            api.append((g1.basis, torch.tensor(kv, device="cuda"),
                        torch.tensor(brng.standard_normal(g1.basis.N), device="cuda"),
                        torch.tensor(brng.standard_normal(g1.basis.N), device="cuda")))

        def api_loop():
            for bm, kt, wv, uv in api:
                kr = kt.clone().requires_grad_(True)
                J = assemble_vjp(k_laplace, bm, wv, uv, k=kr)
                J.backward()
        api_loop()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        api_loop()
        torch.cuda.synchronize()
        ms_api = (time.perf_counter() - t1) * 1e3
        ncell = int(bb.nelems)
        out["batched_512_trip2_forward_vjp"] = {
            "meshes": len(meshes), "nelems": ncell, "nnz": int(ga.entry.nnz), "setup_s": setup_s,
            "step": "CSR values + d(w^T K u)/dk per cell (the coefficient adjoint)",
            "autotuned": best, "ms_graph_replay": ms_graph, "work_units": ga.nunits,
            "ms_union_separate_kernels": ms_union,
            "ms_per_mesh_launches": ms_loop, "ms_per_mesh_launches_one_graph": ms_loop_graph,
            "elements_per_s_batched": ncell / (ms_graph * 1e-3),
            "elements_per_s_per_mesh": ncell / (ms_loop * 1e-3),
            "speedup_vs_per_mesh_launches": ms_loop / ms_graph,
            "speedup_vs_per_mesh_launches_one_graph": ms_loop_graph / ms_graph,
            "ms_per_mesh_api_calls": ms_api, "speedup_vs_per_mesh_api": ms_api / ms_graph,
            "launches_per_step": ga.launches_per_step(),
            "launches_per_step_per_mesh": sum(g.launches_per_step() for g in per)}
        if cpu:
            # the reference's way for many meshes: a Python loop of per-mesh
            # assemblies (forward), on every 16th mesh (their sizes spread as
            # the batch's)
            sample, cells = [], 0
            for mm, kv in list(zip(meshes, ks))[::16]:
                ob = O.OBasis(O.OMesh(np.asarray(mm.p), np.asarray(mm.t), "tri"), O.TriP2())
                sample.append((ob, kv))
                cells += mm.nelements
            c = _cpu_oracle(lambda: [O.bilinear_assemble(O.k_laplace, ob,
                                                         k=ob.zero_w() + kv[:, None],
                                                         nthreads=nthr) for ob, kv in sample],
                            cells, "every 16th mesh (%d meshes, %d cells), a loop of forward "
                                   "assemblies on prebuilt bases" % (len(sample), cells))
            key = "batched_512_trip2_forward_vjp"
            out[key]["cpu_oracle"] = c
            out[key]["speedup_vs_cpu_oracle"] = (out[key]["elements_per_s_batched"] /
                                                 c["cells_per_s"])

    if want("condense"):
        # Dirichlet condensation on the device (skfem.utils.condense,
        # utils.py:462-600): A_II = A[I][:, I] and b_I = b[I] - A[I][:, D] x[D]
        # of the TetP1 k*Laplace+mass system on the --nodes cube, D its
        # boundary nodes; beside it the reference's own scipy slicing of the
        # same system on the host (one run)
        import scipy.sparse as sp
        from skfem_gb300.utils import condense
        n = args.nodes
        m = F.MeshTet.init_tensor(*(np.linspace(0, 1, n),) * 3)
        bs = F.Basis(m, F.ElementTetP1())
        kd = torch.from_numpy(rng.lognormal(0.0, 1.0, m.nelements)).cuda()
        form = k_laplace_mass_form()
        K = form.assemble_torch(bs, k=kd)
        bv = unit_load.assemble_torch(bs)
        D = bs.get_dofs().flatten()
        keep = np.ones(bs.N, dtype=bool)
        keep[D] = False
        I = np.nonzero(keep)[0]
        xv = torch.from_numpy(rng.standard_normal(bs.N)).cuda()
        ms_call = _time(lambda: condense(K, bv, x=xv, D=D), 3, warm=1)
        # the two C-ABI calls alone (map of kept DOFs prebuilt; the pattern
        # call reads back the condensed nnz, one synchronisation)
        mp = np.full(bs.N, -1, dtype=np.int32)
        mp[I] = np.arange(len(I), dtype=np.int32)
        mp_d = torch.from_numpy(mp).cuda()
        crow = K.crow_indices().to(torch.int32).contiguous()
        col = K.col_indices().to(torch.int32).contiguous()
        val = K.values().contiguous()
        oi = torch.empty(len(I) + 1, dtype=torch.int32, device="cuda")
        nnz_c = N.ctypes.c_int64()
        N.check(lib.fem_condense_pattern(N.ptr(crow), N.ptr(col), bs.N, N.ptr(mp_d), len(I),
                                         N.ptr(oi), N.ctypes.byref(nnz_c), N.stream_ptr()))
        oj = torch.empty(max(nnz_c.value, 1), dtype=torch.int32, device="cuda")
        ov = torch.empty(max(nnz_c.value, 1), dtype=torch.float64, device="cuda")
        ob = torch.empty(len(I), dtype=torch.float64, device="cuda")

        def pattern():
            N.check(lib.fem_condense_pattern(N.ptr(crow), N.ptr(col), bs.N, N.ptr(mp_d),
                                             len(I), N.ptr(oi), N.ctypes.byref(nnz_c),
                                             N.stream_ptr()))

        def values():
            N.check(lib.fem_condense_values(N.ptr(crow), N.ptr(col), N.ptr(val), bs.N,
                                            N.ptr(mp_d), N.ptr(bv), N.ptr(xv), N.ptr(oi),
                                            N.ptr(oj), N.ptr(ov), N.ptr(ob), N.stream_ptr()))
        ms_pat = _time(pattern, reps)
        ms_val = _time(values, reps)
        # the same on the host with the reference's slicing, checked against
        # the device result
        Kh = sp.csr_matrix((val.cpu().numpy(), col.cpu().numpy(), crow.cpu().numpy()),
                           shape=(bs.N, bs.N))
        bh, xh = bv.cpu().numpy(), xv.cpu().numpy()
        t0 = time.perf_counter()
        KII = Kh[I][:, I]
        bI = bh[I] - Kh[I][:, D] @ xh[D]
        s_host = time.perf_counter() - t0
        KII.sort_indices()
        AII, bII = condense(K, bv, x=xv, D=D, expand=False)
        same = (np.array_equal(AII.crow_indices().cpu().numpy(), KII.indptr)
                and np.array_equal(AII.col_indices().cpu().numpy(), KII.indices)
                and np.array_equal(AII.values().cpu().numpy(), KII.data))
        b_rel = float(np.abs(bII.cpu().numpy() - bI).max() / np.abs(bI).max())
        # bytes: the CSR read (indptr, indices, values) and the condensed CSR
        # and load vector written
        Bc = (bs.N + 1) * 4 + K.values().numel() * 12 + bs.N * 16 + \
            (len(I) + 1) * 4 + nnz_c.value * 12 + len(I) * 8
        out["condense_tet_p1_%d" % n] = {
            "nrows": int(bs.N), "nnz": int(K.values().numel()), "kept": int(len(I)),
            "nnz_condensed": int(nnz_c.value), "ms_call": ms_call, "ms_pattern": ms_pat,
            "ms_values": ms_val, "gbs_values": Bc / (ms_val * 1e-3) / 1e9,
            "hbm_frac_values": Bc / (ms_val * 1e-3) / 1e9 / hbm,
            "s_host_scipy": s_host, "matches_scipy_bitwise": bool(same),
            "rhs_max_rel_diff": b_rel,
            "step": "condense(K, b, x, D=boundary) on the device CSR; host: the reference's "
                    "A[I][:, I] and b[I] - A[I][:, D] @ x[D] with scipy, one run"}

    if want("generic"):
        # generic per-point kernels: a Newton-step matrix with an
        # interpolated DOF vector (exact reference arithmetic, -fmad=false),
        # and a FacetBasis load on the boundary of the same mesh
        n = args.generic_n
        m = F.MeshTet.init_tensor(*(np.linspace(0, 1, n + 1),) * 3)
        b = F.Basis(m, F.ElementTetP1())
        rng = np.random.default_rng(args.seed)
        s = torch.as_tensor(rng.standard_normal(b.N), device="cuda")

        @F.BilinearForm
        def newton(u, v, w):
            z = w["s"]
            return (1.0 + z ** 2) * H.dot(H.grad(u), H.grad(v)) + 2.0 * z * u * H.dot(
                H.grad(z), H.grad(v))

        @F.LinearForm
        def flux(v, w):
            return H.dot(w.n, w.x) * v

        newton.assemble_torch(b, s=s)                     # pattern built once
        ms_asm = _time(lambda: newton.assemble_torch(b, check=False, s=s), 5)
        ms_interp = _time(lambda: b.interpolate_torch(s), 5)
        ms_local = _time(lambda: newton._local_generic(b, _Coefficients(b, {"s": s})), 5)
        fb = F.FacetBasis(m, F.ElementTetP1())
        flux.assemble_torch(fb)
        ms_facet = _time(lambda: flux.assemble_torch(fb), 5)
        out["generic_newton_tet_p1"] = {
            "nelems": int(b.nelems), "nnz": int(newton.pattern(b, s=s)[1].numel()),
            "ms_assemble": ms_asm, "ms_interpolate": ms_interp,
            "ms_interpolate_plus_local": ms_local,
            "elements_per_s": b.nelems / (ms_asm * 1e-3),
            "facets": int(fb.nelems), "ms_facet_load": ms_facet}

    return out


def cpu_baseline(args, threads=1):
    """The oracle (numpy restatement of the reference) on a bounded sample
    of the workload -- the same form on the 61^3-node cube (1,296,000
    cells) -- timed like scikit-fem's performance.py (Basis construction +
    assemble) and without the Basis (assemble on a prebuilt basis, what the
    GPU step times), on `threads` host threads.  The GPU's CSR of the same
    sample is compared with the oracle's (parity)."""
    import torch

    import oracle as O
    import skfem_gb300 as F
    n = args.cpu_nodes
    m = O.mesh_tet_tensor(*(np.linspace(0, 1, n),) * 3)
    k = np.random.default_rng(SEED).lognormal(0.0, 1.0, m.nelements)
    with_basis, assemble_only = [], []
    Ko = None
    for _ in range(2):
        t0 = time.perf_counter()
        bo = O.OBasis(m, O.TetP1())
        t1 = time.perf_counter()
        Ko = O.bilinear_assemble(O.k_laplace_mass, bo, k=bo.zero_w() + k[:, None], nthreads=threads)
        t2 = time.perf_counter()
        with_basis.append(t2 - t0)
        assemble_only.append(t2 - t1)
    base = {"value": m.nelements / min(assemble_only), "unit": UNIT, "cores": threads,
            "kind": "port",
            "sample": "TetP1 k*laplace+mass on a %d^3-node cube (%d tets), assemble on a prebuilt "
                      "basis, best of 2" % (n, m.nelements),
            "with_basis": {"value": m.nelements / min(with_basis), "unit": UNIT,
                           "sample": "the same, Basis construction + assemble (performance.py)"}}
    # parity: the GPU's CSR of the same sample (host (nelems, nqp) coefficient,
    # public API) against the oracle's
    fm = F.MeshTet(m.p, m.t)
    fb = F.Basis(fm, F.ElementTetP1())
    Kg = k_laplace_mass_form().assemble(fb, k=fb.zero_w() + k[:, None])
    same = (np.array_equal(Kg.indptr, Ko.indptr) and np.array_equal(Kg.indices, Ko.indices))
    rel_fro = rel_max = None
    if same:
        dd = Kg.data - Ko.data
        rel_fro = float(np.linalg.norm(dd) / np.linalg.norm(Ko.data))
        rel_max = float(np.abs(dd).max() / np.abs(Ko.data).max())
    parity = {"against": "oracle (numpy restatement of scikit-fem 12.0.1, pinned to reference "
                         "fixtures)",
              "case": "TetP1 k*laplace+mass, %d^3-node cube, %d cells, nnz %d"
                      % (n, m.nelements, Ko.nnz),
              "indptr_indices_bit_exact": bool(same), "rel_fro": rel_fro, "rel_max": rel_max,
              "bounds": {"rel_fro": 1e-12, "rel_max": 1e-13},
              "ok": bool(same and rel_fro <= 1e-12 and rel_max <= 1e-13)}
    del fb
    torch.cuda.empty_cache()
    return base, parity


def reference_arm(args):
    """The CPU oracle with all host threads on the GPU arm's own workload
    (101^3 nodes, 6M cells): each step assembles on a prebuilt basis, as the
    GPU step does; one Basis + assemble run is reported beside it."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    import oracle as O
    n = args.nodes
    m = O.mesh_tet_tensor(*(np.linspace(0, 1, n),) * 3)
    k = np.random.default_rng(SEED).lognormal(0.0, 1.0, m.nelements)
    t0 = time.perf_counter()
    bo = O.OBasis(m, O.TetP1())
    kw = bo.zero_w() + k[:, None]
    t1 = time.perf_counter()
    O.bilinear_assemble(O.k_laplace_mass, bo, k=kw, nthreads=threads)
    with_basis_s = time.perf_counter() - t0
    basis_s = t1 - t0
    for _ in range(max(0, args.warmup - 1)):
        O.bilinear_assemble(O.k_laplace_mass, bo, k=kw, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.bilinear_assemble(O.k_laplace_mass, bo, k=kw, nthreads=threads)
    dt = (time.perf_counter() - t0) / args.steps
    v = m.nelements / dt
    res = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
           "higher_is_better": True, "scaling": "replicas only", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic (seeded tensor mesh, lognormal k)",
           "config": {"workload": "TetP1 k*laplace+mass, %d^3-node unit cube tensor mesh, 6 "
                                  "tets/cell" % n, "nelems": m.nelements,
                      "step": "assemble on a prebuilt basis (form contraction + COO -> CSR)"},
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": "the whole %d^3-node workload (%d tets) per step"
                                      % (n, m.nelements)},
           "with_basis": {"value": m.nelements / with_basis_s, "unit": UNIT,
                          "basis_s": basis_s, "s": with_basis_s,
                          "note": "one Basis(...) + assemble run, as performance.py times it"},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(res))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nodes", type=int, default=101, help="nodes per axis of the cube")
    ap.add_argument("--cpu-nodes", type=int, default=61, help="nodes per axis of the CPU sample")
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--batch", type=int, default=512, help="meshes of the batched workload")
    ap.add_argument("--vec-n", type=int, default=40, help="cells per axis, vector TetP2 workload")
    ap.add_argument("--p2-n", type=int, default=61,
                    help="nodes per axis, scalar TetP2 workload")
    ap.add_argument("--hex-n", type=int, default=64, help="cells per axis, Hex1 adjoint workload")
    ap.add_argument("--hex-jitter", type=float, nargs="+", default=[0.0, 0.2],
                    help="Hex1 workloads: interior-node jitter (fraction of h) of each case; "
                         "0 = the tensor cube (parallelepiped cells)")
    ap.add_argument("--generic-n", type=int, default=60,
                    help="cells per axis, generic-kernel TetP1 workload")
    ap.add_argument("--only", default=None,
                    choices=["tri_p1", "tet_p2", "tet_p2_vec", "hex1_vjp", "batched",
                             "generic", "condense"],
                    help="run one secondary workload alone and print its record")
    ap.add_argument("--onepass", type=int, default=None, choices=[0, 1, 2],
                    help="fix the one-pass sum's form after autotuning (default: the fastest)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the TriP1 / vector TetP2 / Hex1 adjoint / batched workloads")
    args = ap.parse_args()
    if args.impl == "reference":
        reference_arm(args)
    elif args.only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(secondary_workloads(args, only=args.only)))
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
