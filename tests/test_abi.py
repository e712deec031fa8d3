"""The C-ABI library builds, loads without a GPU, and exports every entry point include/nunatak_gb300.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "nunatak_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nk_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build()
    from nunatak_gb300 import library
    return ctypes.CDLL(library.LIB_PATH)


def test_header_declares_the_solver_entry_points():
    names = declared_functions()
    for n in ("nk_context_create", "nk_problem_create", "nk_picard_solve", "nk_linear_solve", "nk_adjoint_solve",
              "nk_precondition", "nk_apply_operator", "nk_update_coefficients", "nk_compute_geometry"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert missing == []


def test_api_version_without_gpu(lib):
    lib.nk_api_version.restype = ctypes.c_int32
    assert lib.nk_api_version() == 1


def test_descriptor_struct_sizes_match_header():
    """ctypes mirrors of the descriptors have the C layout the library compiles against."""
    from nunatak_gb300 import abi
    assert ctypes.sizeof(abi.IterationControl) == 32
    assert ctypes.sizeof(abi.GridDesc) == 32 + 8 * 2 + 8 * 4 + 8 + 8
    assert ctypes.sizeof(abi.SolverDesc) == 24 + 2 * 32 + 8


def header_defines():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    return {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(NK_[A-Z0-9_]+)\s+(-?\d+)\b", text)}


def test_python_constants_match_the_header():
    """Field ids (including the prescribed velocities) and iteration-control kinds of the ctypes mirror."""
    from nunatak_gb300 import abi
    d = header_defines()
    fields = {k[len("NK_FIELD_"):].lower(): v for k, v in d.items() if k.startswith("NK_FIELD_") and k != "NK_FIELD_COUNT"}
    assert d["NK_FIELD_COUNT"] == len(fields) == len(abi.FIELD_IDS)
    assert sorted(abi.FIELD_IDS.values()) == sorted(fields.values())
    assert abi.FIELD_IDS["u_prescribed"] == d["NK_FIELD_U_PRESCRIBED"] and abi.FIELD_IDS["v_prescribed"] == d["NK_FIELD_V_PRESCRIBED"]
    for name in ("NK_CONVERGENCE", "NK_FIXED_ITERATIONS", "NK_VISCOSITY_CONVERGENCE"):
        assert getattr(abi, name) == d[name]
    assert set(abi.FIELD_LOCATIONS) == set(abi.FIELD_IDS)
