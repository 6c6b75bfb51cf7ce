"""The HDF5 subset (openmc_gb300/csrc/h5lite.cpp and openmc_gb300/h5.py):
the C++ and Python readers agree element by element on files written by
libhdf5 (the reference's data files, when present), by the C++ writer and by
the Python writer; nuclide libraries in OpenMC's incident-neutron HDF5
layout load like the native container; statepoints written through
openmc_statepoint_write read back (CPU only)."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
REF_FILES = ["openmc/data/compton_profiles.h5", "openmc/data/density_effect.h5",
             "tests/regression_tests/random_ray_entropy/mgxs.h5"]


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = tmp_path_factory.mktemp("h5") / "h5lite_check"
    subprocess.run(["g++", "-O1", "-std=c++17", "-o", str(exe), str(ROOT / "tests/native/h5lite_check.cpp"),
                    str(ROOT / "openmc_gb300/csrc/h5lite.cpp")], check=True)
    return exe


def cpp_dump(exe, path):
    r = subprocess.run([str(exe), "dump", str(path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return sorted(r.stdout.splitlines())


def _show(v):
    a = np.asarray(v)
    kind = {"f": "f", "i": "i", "u": "u", "S": "s", "b": "i"}[a.dtype.kind]
    out = f"{kind} ({','.join(str(d) for d in a.shape)})"
    for x in a.reshape(-1):
        if kind == "s":
            out += " '" + bytes(x).split(b"\0")[0].decode() + "'"
        elif kind == "f":
            out += " %.17g" % float(x)
        else:
            out += f" {int(x)}"
    return out


def py_dump(path):
    from openmc_gb300 import h5
    lines = []

    def walk(node, path):
        for k, v in getattr(node, "attrs", {}).items():
            lines.append(f"{path}@{k} A {_show(v)}")
        if isinstance(node, dict):
            lines.append(f"{path} G")
            for name in node:
                walk(node[name], f"{path}/{name}")
        else:
            lines.append(f"{path} D {_show(node)}")

    walk(h5.read(path), "")
    return sorted(lines)


@pytest.mark.parametrize("rel", REF_FILES)
def test_readers_agree_on_libhdf5_files(checker, rel):
    import os
    ref = Path(os.environ.get("OPENMC_REF_ROOT", "/root/reference"))
    path = ref / rel
    if not path.exists():
        pytest.skip("reference data files not present")
    a, b = cpp_dump(checker, path), py_dump(path)
    assert len(a) > 10
    assert a == b


def test_cpp_writer_python_reader(checker, tmp_path):
    path = tmp_path / "w.h5"
    subprocess.run([str(checker), "write", str(path)], check=True)
    assert cpp_dump(checker, path) == py_dump(path)
    from openmc_gb300 import h5
    f = h5.read(path)
    assert len(f["tallies"]) == 150  # two symbol-table nodes
    assert f["tallies/tally 77/results"].tolist() == [[[76.0, 76.0 * 76.0]]]
    assert f["grid"].shape == (3, 4, 2) and f["grid"][2, 3, 1] == 1.0 / 24
    assert f["x"] == -2.5e-300 and int(f["n"]) == 42
    assert f.attrs["version"].tolist() == [18, 1]


def test_python_writer_round_trip(checker, tmp_path):
    from openmc_gb300 import h5
    root = h5.Node({"g": h5.Node({f"m{k:03d}": np.arange(k, dtype=np.int32) for k in range(300)},
                                 {"n": np.int64(300)}),
                    "v": h5.Dataset(np.linspace(0, 1, 7).reshape(7, 1), {"units": np.bytes_(b"eV")}),
                    "s": np.bytes_(b"text"), "u": np.uint64(2 ** 63 + 5), "f32": np.float32([1.5, -2.25])},
                   {"filetype": np.bytes_(b"check"), "pair": np.array([3, 0])})
    path = tmp_path / "p.h5"
    h5.write(path, root)
    f = h5.read(path)
    assert len(f["g"]) == 300
    assert all(f[f"g/m{k:03d}"].tolist() == list(range(k)) for k in range(300))
    assert f["v"].attrs["units"] == b"eV" and np.array_equal(f["v"], np.linspace(0, 1, 7).reshape(7, 1))
    assert int(f["u"]) == 2 ** 63 + 5 and f["f32"].dtype == np.float32
    assert cpp_dump(checker, path) == py_dump(path)


def test_readers_reject_what_they_do_not_read(checker, tmp_path):
    bad = tmp_path / "bad.h5"
    bad.write_bytes(b"\x89HDF\r\n\x1a\n" + b"\xff" * 64)
    r = subprocess.run([str(checker), "dump", str(bad)], capture_output=True, text=True)
    assert r.returncode == 1 and "error" in r.stderr
    from openmc_gb300 import h5
    with pytest.raises(Exception):
        h5.read(bad)


def test_nuclide_h5_layout(checker, tmp_path):
    """write_nuclide_h5 follows the incident-neutron layout
    (docs/source/io_formats/nuclear_data.rst) and both readers see the same
    tables the native container holds."""
    from openmc_gb300 import data, h5
    nuc = data.make_nuclide("U235", 235.0, 400, seed=3, fissile=True)
    path = tmp_path / "U235.h5"
    data.write_nuclide_h5(nuc, path)
    f = h5.read(path)
    assert f.attrs["filetype"] == b"data_neutron" and f.attrs["version"].tolist()[0] == 3
    g = f["U235"]
    assert float(g.attrs["atomic_weight_ratio"]) == nuc.awr
    assert np.array_equal(g["energy/294K"], nuc.energy)
    for mt, (thr, xs) in nuc.reactions.items():
        d = g[f"reactions/reaction_{mt:03d}/294K/xs"]
        assert int(d.attrs["threshold_idx"]) == thr == 0  # 0-based (openmc/data/reaction.py:932-975)
        assert np.array_equal(d, xs)
    assert g["reactions/reaction_018/product_0/distribution_0/energy"].attrs["type"] == b"watt"
    assert cpp_dump(checker, path) == py_dump(path)


def test_h5_library_loads_like_native(built, tmp_path):
    """openmc_init on a cross_sections.xml listing HDF5 nuclide files: the
    model loads with the same nuclides and materials as with the native
    container (the tables themselves are compared by running both on the GPU
    in tests/test_gpu_transport.py)."""
    from openmc_gb300 import configs, lib
    infos = []
    for fmt in ("native", "h5"):
        d = tmp_path / fmt
        d.mkdir()
        m, d = configs.infinite_medium(d, particles=100, batches=3, inactive=1, n_points=200, library_format=fmt)
        m.export_to_model_xml(d / "model.xml")
        lib.init(directory=d)
        try:
            info = (C.c_int64 * 8)()
            lib._dll.openmc_gb300_model_info(info)
            infos.append(list(info))
            mat = lib.materials[m.materials[0].id]
            infos.append(sorted(mat.nuclides))
        finally:
            lib.finalize()
    assert infos[0] == infos[2] and infos[1] == infos[3]


def test_corrupt_h5_library_is_a_data_error(built, tmp_path):
    from openmc_gb300 import configs, lib
    m, d = configs.infinite_medium(tmp_path, particles=100, batches=3, inactive=1, n_points=200,
                                   library_format="h5")
    m.export_to_model_xml(d / "model.xml")
    victim = sorted(Path(d).rglob("*.h5"))[0]
    victim.write_bytes(victim.read_bytes()[:200])
    with pytest.raises(lib.OpenMCError):
        lib.init(directory=d)
    lib.finalize()


def test_statepoint_written_before_transport(built, tmp_path):
    """openmc_statepoint_write after openmc_init: run parameters, meshes,
    filters and tallies as the model gives them; zero results."""
    from openmc_gb300 import configs, lib
    from openmc_gb300.statepoint import StatePoint
    m, d = configs.lattice17(tmp_path, particles=100, batches=3, n_points=300, mesh_dim=(17, 17, 5), n_ebins=4)
    m.export_to_model_xml(d / "model.xml")
    lib.init(directory=d)
    try:
        lib.statepoint_write(d / "sp.h5")
        with pytest.raises(lib.OpenMCError):
            lib.statepoint_write(d / "no_such_dir" / "sp.h5")
    finally:
        lib.finalize()
    sp = StatePoint(d / "sp.h5")
    assert sp.version == (18, 1) and sp.run_mode == "fixed source"
    assert sp.n_particles == 100 and sp.n_batches == 3 and sp.current_batch == 0 and sp.n_realizations == 0
    assert sp.seed >= 1 and sp.stride == 152917
    assert set(sp.tallies) == {t.id for t in m.tallies}
    for t in m.tallies:
        st = sp.tallies[t.id]
        assert [f.id for f in st.filters] == [f.id for f in t.filters]
        assert np.all(st.sum == 0) and st.sum.shape[1:] == (1, len(t.scores))
        assert st.sum.shape[0] == int(np.prod([f.num_bins for f in st.filters]))
    mesh = next(iter(sp.meshes.values()))
    assert mesh.dimension == (17, 17, 5)
    assert np.all(sp.global_tallies["sum"] == 0)


def test_reader_survives_corrupt_files(checker, tmp_path):
    """Truncated and byte-flipped copies of a nuclide file make the C++
    reader report an error (or read what is still valid), never crash:
    every read is bounds-checked and every walk bounded."""
    from openmc_gb300 import data
    nuc = data.make_nuclide("U235", 235.0, 200, seed=3, fissile=True)
    good = tmp_path / "good.h5"
    data.write_nuclide_h5(nuc, good)
    raw = bytearray(good.read_bytes())
    rng = np.random.default_rng(17)
    cases = [bytes(raw[:n]) for n in sorted(set(rng.integers(0, len(raw), 40).tolist()))]
    for _ in range(120):
        b = bytearray(raw)
        for pos in rng.integers(0, len(b), int(rng.integers(1, 6))):
            b[pos] = int(rng.integers(0, 256))
        cases.append(bytes(b))
    for k, c in enumerate(cases):
        f = tmp_path / f"bad{k}.h5"
        f.write_bytes(c)
        r = subprocess.run([str(checker), "dump", str(f)], capture_output=True, timeout=60)
        assert r.returncode in (0, 1), (k, r.returncode, r.stderr[-300:].decode(errors="replace"))


def test_truncated_native_nuclide_is_an_error(built, tmp_path):
    """The native container's reader checks every read against the file's
    size: truncated copies fail at openmc_init with a message, never crash."""
    import subprocess as sp
    import sys
    from openmc_gb300 import configs
    m, d = configs.infinite_medium(tmp_path, particles=100, batches=3, inactive=1, n_points=200)
    m.export_to_model_xml(d / "model.xml")
    victim = sorted(Path(d).rglob("*.nuc"))[0]
    raw = victim.read_bytes()
    script = ("import sys\n"
              "from openmc_gb300 import lib\n"
              "try:\n"
              "    lib.init(directory=sys.argv[1])\n"
              "except lib.OpenMCError as e:\n"
              "    print('error', e)\n"
              "lib.finalize()\n")
    for n in (20, 60, len(raw) // 3, len(raw) - 9):
        victim.write_bytes(raw[:n])
        r = sp.run([sys.executable, "-c", script, str(d)], capture_output=True, text=True, cwd=str(ROOT), timeout=120)
        assert r.returncode == 0 and "error" in r.stdout, (n, r.returncode, r.stdout[-200:], r.stderr[-300:])
