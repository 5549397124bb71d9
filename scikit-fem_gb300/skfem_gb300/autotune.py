"""Autotuner of the launch parameters (cells per CTA of the local kernel,
persistent grid, incidence entries loaded together by the segmented sum,
and for the scalar bases with an even number of local functions the
columns per lane of the fused sum).

Times ``fem_assemble`` on the caller's own basis and form for every
candidate (CUDA events, after warm-up), keeps the fastest and sets it with
``fem_set_tuning``.  Results are cached in a JSON file keyed by GPU, element
family, vector flag and problem size class.
"""

import itertools
import json
import os

import torch

from . import _native as N

CANDIDATES = {
    "local_block": (64, 128, 256),
    "persistent": (0, 4),
    "sum_unroll": (4, 8, 16),
}
# columns per lane of the fused sum: the scalar bases with 4, 6 or 10 local
# functions also have the two-columns-per-lane kernel
COLS = {"TetP1": (1, 2), "TriP2": (1, 2), "TetP2": (1, 2)}
# the one-pass P1 sum's forms (two lanes per row / a lane per upper entry /
# the same with TMA-staged list codes), which give the same bits; for the
# scalar P2 families the one-pass node-block sum's two forms (per
# contribution / one FMA per step), also bitwise equal -- their two-pass
# alternative adds in another grouping and is never tried: a tuning never
# changes the values
ONEPASS = {"TriP1": (0, 1, 2), "TetP1": (0, 1, 2), "TriP2": (1, 2), "TetP2": (1, 2)}


def candidates(family, vector=False):
    """Every configuration the autotuner times for a basis of this family:
    the product of CANDIDATES, times the columns per lane of the fused sum
    where the family has the two-columns kernel, times the one-pass sum's
    forms for the simplex families (scalar bases only)."""
    cols = (1,) if vector else COLS.get(family, (1,))
    onep = (1,) if vector else ONEPASS.get(family, (1,))
    return [{"local_block": lb, "persistent": pers, "sum_unroll": un, "sum_cols": nc,
             "onepass": op}
            for lb, pers, un, nc, op in itertools.product(*CANDIDATES.values(), cols, onep)]


def _cache_path():
    root = os.environ.get("SKFEM_GB300_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "skfem_gb300"))
    os.makedirs(root, exist_ok=True)
    return os.path.join(root, "autotune.json")


def _key(basis):
    name = torch.cuda.get_device_name(basis.device)
    size = int(basis.nelems).bit_length()
    return "%s|%s|%d|%d" % (name, basis.elem.family, int(basis.elem.vector), size)


def apply(family_code, cfg):
    N.check(N.lib().fem_set_tuning(family_code, cfg["local_block"], cfg["persistent"],
                                   cfg["sum_unroll"], cfg.get("sum_cols", 1)))
    N.check(N.lib().fem_set_onepass(family_code, cfg.get("onepass", 1)))


def tune(form, basis, coefs, reps=3, use_cache=True):
    """Pick and apply the fastest launch configuration; returns (cfg, timings)."""
    fam = N.FAMILY[basis.elem.family]
    path = _cache_path()
    cache = {}
    if os.path.exists(path):
        try:
            cache = json.load(open(path))
        except ValueError:
            cache = {}
    key = _key(basis)
    if use_cache and key in cache:
        apply(fam, cache[key]["best"])
        return cache[key]["best"], cache[key]["timings"]
    form.assemble_torch(basis, **coefs)
    entry = next(e for k, e in basis._patterns.items() if k[0] == "bilinear")
    _, _, c_form = form._setup(basis, None, coefs)
    vals = torch.empty(entry.nnz, dtype=torch.float64, device=basis.device)
    # a status word, as assemblies pass one (the TMA-staged one-pass form
    # runs only with it)
    status = torch.zeros(1, dtype=torch.int32, device=basis.device)
    lib = N.lib()
    timings = []
    for cfg in candidates(basis.elem.family, bool(basis.elem.vector)):
        apply(fam, cfg)
        s = N.stream_ptr()

        def step():
            N.check(lib.fem_assemble(N.byref(basis.c_mesh), N.byref(basis.c_basis),
                                     N.byref(c_form), entry.pat.handle, N.ptr(entry.staging),
                                     N.ptr(vals), N.ptr(status), s))
        step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            step()
        e1.record()
        torch.cuda.synchronize()
        timings.append((e0.elapsed_time(e1) / reps, cfg))
    timings.sort(key=lambda x: x[0])
    best = timings[0][1]
    apply(fam, best)
    cache[key] = {"best": best, "timings": [[t, c] for t, c in timings]}
    try:
        json.dump(cache, open(path, "w"), indent=1)
    except OSError:
        pass
    return best, timings
