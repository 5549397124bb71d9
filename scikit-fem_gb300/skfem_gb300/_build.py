"""In-tree build of libskfem_gb300.so for sm_103a (GB300).

The translation units of UNITS compiled in parallel with one -gencode each;
the local-matrix kernels are compiled twice: with FMA contraction (values)
and with ``-fmad=false`` (the exact-zero mask of the pattern build).  The
header texts the run-time compiler embeds (fem_jit_sources.inc) are written
into the output folder on every build, never committed.
"""

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libskfem_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills"]

UNITS = [
    ("fem_local.cu", "fem_local_fast.o", []),
    ("fem_local.cu", "fem_local_exact.o", ["-DFEM_EXACT", "-fmad=false"]),
    ("fem_pattern.cu", "fem_pattern.o", []),
    ("fem_vjp.cu", "fem_vjp.o", []),
    ("fem_batched.cu", "fem_batched.o", []),
    ("fem_vecsum.cu", "fem_vecsum.o", []),
    ("fem_abi.cu", "fem_abi.o", []),
    ("fem_noalloc.cu", "fem_noalloc.o", []),
    ("fem_faithful.cu", "fem_faithful.o", ["-fmad=false"]),
    ("fem_condense.cu", "fem_condense.o", []),
    ("fem_jit.cu", "fem_jit.o", ["-I", OUT_DIR]),
]

# headers the run-time compiler of form programs needs, embedded as text
JIT_SOURCES = [("kJitCoreSrc", os.path.join(CSRC, "fem_faithful_core.cuh")),
               ("kJitKernelSrc", os.path.join(CSRC, "fem_program_kernel.cuh")),
               ("kJitAbiSrc", os.path.join(os.path.dirname(ROOT), "include", "skfem_gb300.h"))]


def write_jit_sources():
    out = ["// Generated by skfem_gb300/_build.py: header texts for fem_jit.cu."]
    for name, path in JIT_SOURCES:
        text = open(path).read()
        if ")FEMSRC\"" in text:
            raise RuntimeError("raw-string delimiter found in %s" % path)
        out.append('static const char* %s = R"FEMSRC(%s)FEMSRC";' % (name, text))
    tmp = os.path.join(OUT_DIR, "fem_jit_sources.inc.tmp")
    open(tmp, "w").write("\n".join(out) + "\n")
    os.replace(tmp, os.path.join(OUT_DIR, "fem_jit_sources.inc"))


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the skfem_gb300 CUDA library cannot be built")


def _sources_newer_than(path):
    if not os.path.exists(path):
        return True
    t = os.path.getmtime(path)
    for f in os.listdir(CSRC):
        if f.endswith((".cu", ".cuh", ".h")) and os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    hdr = os.path.join(os.path.dirname(ROOT), "include", "skfem_gb300.h")
    return os.path.exists(hdr) and os.path.getmtime(hdr) > t


def build(force=False, verbose=False):
    """Compile the CUDA library if any source changed; returns the .so path."""
    if not force and not _sources_newer_than(LIB):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    # fem_tables.cuh / fem_refquad.cuh are generated once by gen_tables.py /
    # gen_refquad.py and committed: regenerating them on another platform
    # could change the last bits of numpy-computed quadrature nodes.
    cc = nvcc()
    write_jit_sources()
    missing = [u[0] for u in UNITS if not os.path.exists(os.path.join(CSRC, u[0]))]
    if missing:
        raise RuntimeError("missing CUDA sources: %s" % ", ".join(missing))
    units = UNITS

    def compile_unit(u):
        src, obj, extra = u
        cmd = [cc] + ARCH + FLAGS + extra + ["-c", os.path.join(CSRC, src), "-o",
                                             os.path.join(OUT_DIR, obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        return r.stderr

    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        logs = list(ex.map(compile_unit, units))
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + [os.path.join(OUT_DIR, u[1]) for u in units] + [
        "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
