"""The C ABI library builds, loads and exports every declared entry point;
no compute call is made (no GPU here)."""
import ctypes

import pytest


def test_library_exports_header_symbols(built):
    from trimem_gb300 import capi

    names = capi.header_functions()
    assert len(names) >= 40
    lib = ctypes.CDLL(capi.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_header(built):
    from trimem_gb300 import capi

    assert set(capi.header_functions()) <= set(capi._SIGS)


def test_pybind_module_imports_and_exposes_reference_api(built):
    from trimem_gb300 import load_core

    m = load_core()
    for name in ["TriMesh", "HalfedgeHandle", "VertexProperties", "BondType", "BondParams",
                 "SurfaceRepulsionParams", "ContinuationParams", "EnergyParams", "EnergyManager",
                 "NeighbourList", "Point", "read_mesh", "edge_length", "edge_length_grad", "face_area",
                 "face_area_grad", "face_volume", "face_volume_grad", "dihedral_angle",
                 "dihedral_angle_grad", "flip", "pflip", "make_nlist", "area", "edges_length",
                 "avg_tri_props", "gradient"]:
        assert hasattr(m, name), name
    p = m.EnergyParams()
    assert p.area_frac == 1 and p.repulse_params.n_search == "cell-list"
    assert p.repulse_params.rlist == pytest.approx(0.1) and p.bond_params.r == 2
    assert p.continuation_params.lam == 1


def test_params_struct_layout_matches_header(built):
    from trimem_gb300 import capi

    assert ctypes.sizeof(capi.Params) == 8 * 12 + 4 * 2 + 8 + 4 * 2 + 8 + 4 * 2 + 8 * 2
