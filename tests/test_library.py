"""The C-ABI library: loads, exports every symbol include/*.h declares and
every function and global the reference's Python bindings resolve, parses
models, answers model queries and reports errors like the reference (CPU
only; no compute calls)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def header_symbols():
    text = "".join(h.read_text() for h in sorted((ROOT / "include").glob("*.h")))
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


def test_reference_bindings_resolve(built):
    """openmc/lib/*.py declares argument types for every function it uses at
    import, so each must be exported for `import openmc.lib` to succeed on
    this library (list generated by tests/golden/make_bindings_list.py)."""
    import json
    from openmc_gb300 import lib
    names = json.loads((ROOT / "tests" / "golden" / "openmc_lib_bindings.json").read_text())
    assert len(names["functions"]) > 150 and len(names["globals"]) > 15
    dll = C.CDLL(lib.loaded_library())
    missing = [f for f in names["functions"] if not hasattr(dll, f)]
    assert not missing, f"functions the reference's bindings need: {missing}"
    for g in names["globals"]:
        C.c_int.in_dll(dll, g)


def test_model_queries_and_off_path_calls(built, tmp_path):
    from openmc_gb300 import configs, lib
    m, d = configs.lattice17(tmp_path, particles=100, batches=3, n_points=300, mesh_dim=(17, 17, 5), n_ebins=4)
    m.export_to_model_xml(d)
    lib.init(directory=d)
    try:
        # a separate handle: return codes as the reference's bindings see them
        dll = C.CDLL(lib.loaded_library())

        def code(name):
            return C.c_int.in_dll(dll, "OPENMC_E_" + name).value

        i32, i = C.c_int32(), C.c_int()
        tally = m.tallies[0]
        mesh_f, energy_f = tally.filters
        # filters: index by id, type, bins
        assert dll.openmc_get_filter_index(mesh_f.id, C.byref(i32)) == 0
        fi = i32.value
        buf = C.create_string_buffer(32)
        assert dll.openmc_filter_get_type(fi, buf) == 0 and buf.value == b"mesh"
        assert dll.openmc_mesh_filter_get_mesh(fi, C.byref(i32)) == 0
        mi = i32.value
        assert dll.openmc_get_filter_index(energy_f.id, C.byref(i32)) == 0
        ei = i32.value
        e_ptr, n = C.POINTER(C.c_double)(), C.c_size_t()
        assert dll.openmc_energy_filter_get_bins(ei, C.byref(e_ptr), C.byref(n)) == 0
        assert n.value == 5 and e_ptr[0] < e_ptr[4]
        assert dll.openmc_energy_filter_get_bins(fi, C.byref(e_ptr), C.byref(n)) == code("INVALID_TYPE")
        # the regular mesh's dimension and parameters (borrowed pointers)
        dims, nd = C.POINTER(C.c_int)(), C.c_int()
        assert dll.openmc_regular_mesh_get_dimension(mi, C.byref(dims), C.byref(nd)) == 0
        assert [dims[k] for k in range(nd.value)] == [17, 17, 5]
        ll, ur, w = C.POINTER(C.c_double)(), C.POINTER(C.c_double)(), C.POINTER(C.c_double)()
        assert dll.openmc_regular_mesh_get_params(mi, C.byref(ll), C.byref(ur), C.byref(w), C.byref(nd)) == 0
        assert np.isclose(ur[0] - ll[0], 17 * w[0])
        assert dll.openmc_mesh_get_type(mi, buf) == 0 and buf.value == b"regular"
        # tallies: estimator (TallyEstimator::TRACKLENGTH), flux score code, filters
        ti = lib.tally_index(tally.id)
        assert dll.openmc_tally_get_estimator(ti, C.byref(i)) == 0 and i.value == 1
        sc, ns = C.POINTER(C.c_int)(), C.c_int()
        assert dll.openmc_tally_get_scores(ti, C.byref(sc), C.byref(ns)) == 0 and ns.value == 1 and sc[0] == -1
        fl, nf = C.POINTER(C.c_int32)(), C.c_size_t()
        assert dll.openmc_tally_get_filters(ti, C.byref(fl), C.byref(nf)) == 0
        assert [fl[k] for k in range(nf.value)] == [fi, ei]
        # cells and materials by id; an unknown id
        cid = m.geometry.root_universe.cells[0].id
        assert dll.openmc_get_cell_index(cid, C.byref(i32)) == 0
        out = C.c_int32()
        assert dll.openmc_cell_get_id(i32.value, C.byref(out)) == 0 and out.value == cid
        assert dll.openmc_get_material_index(99999, C.byref(i32)) == code("INVALID_ID")
        # the root cell is filled with the lattice (Fill::LATTICE = 2)
        ft, fidx, fn = C.c_int(), C.POINTER(C.c_int32)(), C.c_int32()
        assert dll.openmc_get_cell_index(cid, C.byref(i32)) == 0
        assert dll.openmc_cell_get_fill(i32.value, C.byref(ft), C.byref(fidx), C.byref(fn)) == 0
        assert ft.value == 2 and fn.value == 1 and fidx[0] == 0
        # instances (one per lattice position of the pin universe) and boxes
        lat = m.geometry.root_universe.cells[0].fill
        fuel_cell = lat.universes[0][0].cells[0]
        guide_water = lat.universes[2][5].cells[0]
        ni = C.c_int32()
        for cell, expect in ((fuel_cell, 17 * 17 - 25), (guide_water, 25), (m.geometry.root_universe.cells[0], 1)):
            assert dll.openmc_get_cell_index(cell.id, C.byref(i32)) == 0
            assert dll.openmc_cell_get_num_instances(i32.value, C.byref(ni)) == 0 and ni.value == expect
        llc, urc = (C.c_double * 3)(), (C.c_double * 3)()
        assert dll.openmc_global_bounding_box(llc, urc) == 0
        assert np.allclose(list(llc), [-10.71, -10.71, -100.0]) and np.allclose(list(urc), [10.71, 10.71, 100.0])
        assert dll.openmc_get_cell_index(fuel_cell.id, C.byref(i32)) == 0
        assert dll.openmc_cell_bounding_box(i32.value, llc, urc) == 0
        assert np.allclose(list(llc)[:2], [-0.41, -0.41]) and np.allclose(list(urc)[:2], [0.41, 0.41])
        assert np.isinf(llc[2]) and np.isinf(urc[2])
        # a material's nuclides and atom densities (borrowed), and its mass density
        mat = m.materials[0]
        assert dll.openmc_get_material_index(mat.id, C.byref(i32)) == 0
        nuc, dens, nn = C.POINTER(C.c_int)(), C.POINTER(C.c_double)(), C.c_int()
        assert dll.openmc_material_get_densities(i32.value, C.byref(nuc), C.byref(dens), C.byref(nn)) == 0
        assert nn.value == 4 and all(dens[k] > 0 for k in range(4))
        rho = C.c_double()
        assert dll.openmc_material_get_density(i32.value, C.byref(rho)) == 0 and rho.value > 0
        name = C.c_char_p()
        assert dll.openmc_nuclide_name(nuc[0], C.byref(name)) == 0
        back = C.c_int()
        assert dll.openmc_get_nuclide_index(name.value, C.byref(back)) == 0 and back.value == nuc[0]
        # batches and k (fixed source: 1 with an infinite spread before two realizations)
        assert dll.openmc_get_n_batches(C.byref(i), False) == 0 and i.value == 3
        k = (C.c_double * 2)()
        assert dll.openmc_get_keff(k) == 0 and k[0] == 1.0 and np.isinf(k[1])
        # an entry point outside the path: an error code and a message, no crash
        assert dll.openmc_calculate_volumes() == code("UNASSIGNED")
        assert b"openmc_calculate_volumes" in (C.c_char * 256).in_dll(dll, "openmc_err_msg").value
    finally:
        lib.finalize()


def test_python_model_views(built, tmp_path):
    """openmc.lib-style views of the loaded model: cells, materials and
    meshes keyed by id, global bounding box, k-effective."""
    from openmc_gb300 import configs, lib
    m, d = configs.lattice17(tmp_path, particles=100, batches=3, n_points=300, mesh_dim=(17, 17, 5), n_ebins=4)
    m.export_to_model_xml(d)
    lib.init(directory=d)
    try:
        root = m.geometry.root_universe.cells[0]
        lat = root.fill
        assert len(lib.cells) == 1 + 3 + 3 and root.id in lib.cells.keys()
        assert lib.cells[root.id].fill == ("lattice", 0)
        assert lib.cells[lat.universes[0][0].cells[0].id].num_instances == 17 * 17 - 25
        lo, hi = lib.global_bounding_box()
        assert np.allclose(lo, [-10.71, -10.71, -100.0]) and np.allclose(hi, [10.71, 10.71, 100.0])
        with pytest.raises(KeyError):
            lib.cells[987654]
        fuel = lib.materials[m.materials[0].id]
        assert fuel.nuclides == ["Hv235", "Hv238", "Ox16", "Hv240"]
        assert np.isclose(fuel.densities.sum(), 0.069) and fuel.get_density() > 0
        mesh = lib.meshes[m.tallies[0].filters[0].mesh.id]
        assert mesh.dimension == (17, 17, 5)
        assert np.allclose(mesh.upper_right - mesh.lower_left, [17 * 1.26, 17 * 1.26, 200.0])
        assert np.allclose(mesh.width * np.array(mesh.dimension), mesh.upper_right - mesh.lower_left)
        assert len(lib.meshes) == 1
        k, s = lib.keff()
        assert k == 1.0 and np.isinf(s)
    finally:
        lib.finalize()


@pytest.mark.parametrize("case", ["survival_biasing", "generations_per_batch"])
def test_unsupported_settings_rejected(built, tmp_path, case):
    """Settings the GPU path does not implement fail at openmc_init instead
    of running without them."""
    from openmc_gb300 import configs, lib
    m, d = configs.point_cube(tmp_path, particles=100, batches=2, n_points=300, mesh_dim=(2, 2, 2), n_ebins=2)
    if case == "survival_biasing":
        m.settings.survival_biasing = True
    else:
        m.settings.run_mode = "eigenvalue"
        m.settings.generations_per_batch = 2
    m.export_to_model_xml(d)
    with pytest.raises(lib.InvalidArgumentError):
        lib.init(directory=d)
    lib.finalize()
