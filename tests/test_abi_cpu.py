"""CPU checks of the C ABI: the library builds for sm_103a, loads, and
exports every function include/skfem_gb300.h declares (no compute calls)."""
import ctypes

from _util import header_functions


def test_header_declares_entry_points():
    fns = header_functions()
    for f in ("fem_pattern_build", "fem_assemble", "fem_bilinear_vjp", "fem_last_error"):
        assert f in fns


def test_library_exports_every_declared_symbol():
    from skfem_gb300 import _build
    path = _build.build()
    lib = ctypes.CDLL(path)
    missing = [f for f in header_functions() if not hasattr(lib, f)]
    assert not missing, missing
    lib.fem_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.fem_version()
    lib.fem_last_error.restype = ctypes.c_char_p
    assert lib.fem_last_error() == b""


def test_argument_errors_without_gpu():
    """Validation happens on the host before any CUDA call."""
    from skfem_gb300 import _build, _native as N
    lib = ctypes.CDLL(_build.build())
    lib.fem_last_error.restype = ctypes.c_char_p
    m = N.FemMesh(2, 3, 4, 2, None, None)
    b = N.FemBasis(N.FAMILY["TetP1"], 0, 4, 0, 4, None)  # 3-D element on a 2-D mesh
    f = N.FemBilinear()
    rc = lib.fem_local_matrices(ctypes.byref(m), ctypes.byref(b), ctypes.byref(f), None, None)
    assert rc == N.FEM_ERR_ARGUMENT
    assert b"Incompatible Mesh and Element" in lib.fem_last_error()
    b = N.FemBasis(99, 0, 4, 0, 4, None)
    rc = lib.fem_local_matrices(ctypes.byref(m), ctypes.byref(b), ctypes.byref(f), None, None)
    assert rc == N.FEM_ERR_UNSUPPORTED


def test_pipeline_and_cache_entry_points_validate_on_the_host():
    """The host-pipelined assembly and the geometry cache refuse bad
    arguments before any CUDA call."""
    from skfem_gb300 import _build, _native as N
    lib = ctypes.CDLL(_build.build())
    lib.fem_last_error.restype = ctypes.c_char_p
    m = N.FemMesh(3, 4, 4, 1, None, None)
    b = N.FemBasis(N.FAMILY["TetP1"], 0, 4, 0, 4, None)
    f = N.FemBilinear()
    V = ctypes.c_void_p
    # null pattern / buffers
    lib.fem_assemble_to_host_pipelined.argtypes = [V] * 8 + [V, ctypes.c_int32, ctypes.c_int32,
                                                             V, V, V]
    rc = lib.fem_assemble_to_host_pipelined(ctypes.addressof(m), ctypes.addressof(b),
                                            ctypes.addressof(f), None, None, None, None, None,
                                            None, 0, 8, None, None, None)
    assert rc == N.FEM_ERR_ARGUMENT
    # chunk count out of range, host rows announced but not given
    for nfields, nchunks in ((0, 0), (0, 257), (2, 8), (17, 8)):
        rc = lib.fem_assemble_to_host_pipelined(ctypes.addressof(m), ctypes.addressof(b),
                                                ctypes.addressof(f), None, None, None, None,
                                                None, None, nfields, nchunks, None, None, None)
        assert rc == N.FEM_ERR_ARGUMENT
    lib.fem_pattern_cache_geometry.argtypes = [V, V, V, V]
    rc = lib.fem_pattern_cache_geometry(None, ctypes.addressof(m), ctypes.addressof(b), None)
    assert rc == N.FEM_ERR_ARGUMENT
    lib.fem_pattern_drop_geometry.argtypes = [V]
    lib.fem_pattern_drop_geometry(None)          # null: a no-op


def test_staged_sum_validates_on_the_host():
    """fem_csr_sum_staged (the sum half of fem_assemble in the pattern's
    staging layout) refuses a null pattern before any CUDA call."""
    from skfem_gb300 import _build, _native as N
    lib = ctypes.CDLL(_build.build())
    lib.fem_last_error.restype = ctypes.c_char_p
    V = ctypes.c_void_p
    lib.fem_csr_sum_staged.argtypes = [V, V, V, V]
    rc = lib.fem_csr_sum_staged(None, None, None, None)
    assert rc == N.FEM_ERR_ARGUMENT
    assert b"null pattern" in lib.fem_last_error()


def test_tuning_is_validated_on_the_host():
    """fem_set_tuning refuses values outside its documented sets (block
    64/128/256, unroll 4/8/16, columns per lane 1/2) and accepts the rest;
    no CUDA call is involved."""
    from skfem_gb300 import _build, _native as N
    lib = ctypes.CDLL(_build.build())
    fam = N.FAMILY["TetP1"]
    for bad in ((fam, 96, 0, 8, 1), (fam, 128, -1, 8, 1), (fam, 128, 0, 5, 1),
                (fam, 128, 0, 8, 3), (0, 128, 0, 8, 1), (9, 128, 0, 8, 1)):
        assert lib.fem_set_tuning(*bad) == N.FEM_ERR_ARGUMENT
    assert lib.fem_set_tuning(fam, 128, 0, 8, 2) == 0
    assert lib.fem_set_tuning(fam, 128, 0, 8, 1) == 0


def test_onepass_variant_is_validated_on_the_host():
    """fem_set_onepass takes variants 0-2 for families 1-5 and refuses the
    rest; no CUDA call."""
    from skfem_gb300 import _build, _native as N
    lib = ctypes.CDLL(_build.build())
    fam = N.FAMILY["TetP1"]
    for bad in ((fam, -1), (fam, 3), (0, 1), (6, 1)):
        assert lib.fem_set_onepass(*bad) == N.FEM_ERR_ARGUMENT
    for v in (0, 2, 1):
        assert lib.fem_set_onepass(fam, v) == 0
