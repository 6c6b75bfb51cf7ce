"""The C-ABI library: loads, exports every symbol include/openmc_gb300.h
declares, parses models and reports errors like the reference (CPU only; no
compute calls)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def header_symbols():
    text = (ROOT / "include" / "openmc_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    funcs = re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b((?:openmc_|tallies_)\w+)\s*\(", text, flags=re.M)
    globs = re.findall(r"^\s*extern\s+[\w\s\*]+?\b(\w+)(?:\[\d+\])?\s*;", text, flags=re.M)
    return sorted(set(funcs)), sorted(set(globs))


def test_exports_every_declared_symbol(built):
    from openmc_gb300 import lib
    funcs, globs = header_symbols()
    assert len(funcs) > 30 and len(globs) > 20
    dll = C.CDLL(lib.loaded_library())
    missing = [s for s in funcs + globs if not hasattr(dll, s)]
    assert not missing, f"symbols declared but not exported: {missing}"


def test_error_before_init(built):
    from openmc_gb300 import lib
    lib.finalize()
    with pytest.raises(lib.AllocationError):
        lib.simulation_init()
    with pytest.raises(lib.AllocationError):
        lib.next_batch()


def test_bad_model_path(built, tmp_path):
    from openmc_gb300 import lib
    with pytest.raises(lib.InvalidArgumentError):
        lib.init(directory=tmp_path / "nowhere")
    lib.finalize()


def test_init_parses_model(built, tmp_path):
    from openmc_gb300 import configs, lib
    from oracle import flatten
    m, d = configs.lattice17(tmp_path, particles=100, batches=3, n_points=300, mesh_dim=(17, 17, 5), n_ebins=4)
    xml = m.export_to_model_xml(d)
    lib.init(directory=d)
    try:
        info = (C.c_int64 * 8)()
        lib._dll.openmc_gb300_model_info(info)
        a = flatten.load_model(xml)
        assert info[0] == len(a["nuc_off"]) - 1
        assert info[1] == len(a["mat_id"])
        assert info[2] == len(a["cell_id"])
        assert info[3] == len(a["surf_type"])
        assert info[7] == 2  # lattice -> pin universe
        assert lib.settings.particles == 100
        lib.settings.particles = 50
        assert lib.settings.particles == 50
        assert lib.tally_index(m.tallies[0].id) == 0
        with pytest.raises(lib.InvalidIDError):
            lib.tally_index(999)
    finally:
        lib.finalize()


def test_weight_window_api(built, tmp_path):
    from openmc_gb300 import configs, lib
    from openmc_gb300 import model as om
    mesh = om.RegularMesh()
    mesh.dimension = [20, 1, 1]
    mesh.lower_left = [0.0, -25.0, -25.0]
    mesh.upper_right = [200.0, 25.0, 25.0]
    lower = np.exp(-0.3 * np.arange(20))
    ww = om.WeightWindows(mesh, lower, upper_bound_ratio=5.0, energy_bounds=[0.0, 2.0e7])
    m, d = configs.shield(tmp_path, particles=100, batches=2, n_points=300, mesh_dim=(20, 1, 1),
                          weight_windows=ww)
    m.export_to_model_xml(d)
    lib.init(directory=d)
    try:
        assert lib.weight_windows_size() == 1
        assert lib.settings.weight_windows_on
        w = lib.WeightWindows(0)
        lo, up = w.bounds
        assert np.allclose(lo, lower) and np.allclose(up, 5.0 * lower)
        w.bounds = (lo * 2, up * 2)
        assert np.allclose(w.bounds[0], 2 * lower)
        with pytest.raises(lib.InvalidArgumentError):
            w.bounds = (lo[:3], up[:3])
        assert np.allclose(w.energy_bounds, [0.0, 2.0e7])
    finally:
        lib.finalize()


def test_no_cpu_fallback(built, tmp_path):
    """Without a GPU, simulation_init fails loudly instead of falling back."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from openmc_gb300 import configs, lib
    m, d = configs.point_cube(tmp_path, particles=10, batches=1, n_points=100)
    m.export_to_model_xml(d)
    lib.init(directory=d)
    try:
        with pytest.raises(lib.OpenMCError):
            lib.simulation_init()
    finally:
        lib.finalize()


@pytest.mark.parametrize("case", ["analog", "unknown_cell", "two_cell_filters"])
def test_unsupported_tallies_rejected(built, tmp_path, case):
    """Tally options outside the GPU path fail at openmc_init with an
    OPENMC_E_INVALID_ARGUMENT message, as the reference's input checks do."""
    from openmc_gb300 import configs, lib
    from openmc_gb300 import model as om
    m, d = configs.point_cube(tmp_path, particles=100, batches=2, n_points=300, mesh_dim=(2, 2, 2), n_ebins=2)
    t = om.Tally(name="bad")
    cells = m.geometry.root_universe.cells
    if case == "analog":
        t.estimator = "analog"
    elif case == "unknown_cell":
        t.filters = [om.CellFilter([987654])]
    else:
        t.filters = [om.CellFilter(cells[:1]), om.CellFilter(cells[1:])]
    m.tallies.append(t)
    m.export_to_model_xml(d)
    with pytest.raises(lib.InvalidArgumentError):
        lib.init(directory=d)
    lib.finalize()
