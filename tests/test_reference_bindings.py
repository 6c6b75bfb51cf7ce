"""The reference's own Python bindings (openmc/lib/*.py, unmodified) drive
this library: with the package importable (its missing third-party
dependencies, none of which openmc.lib uses, replaced by empty modules) and
the one switch of the drop-in boundary applied (CDLL of openmc/lib's
libopenmc.so opens this library instead), openmc.lib initialises a model and
answers through its own classes (CPU only: no transport).  Skipped when the
reference tree is absent."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
REF = Path(os.environ.get("OPENMC_REF_ROOT", "/root/reference"))

SCRIPT = r'''
import ctypes, importlib.abc, importlib.machinery, importlib.metadata, json, sys, types
ref, lib_path, model_dir = sys.argv[1:4]

# the reference package imports these at top level; openmc.lib does not use them
STUBS = ("h5py", "lxml", "pandas", "uncertainties", "matplotlib", "endf")
class Stub(types.ModuleType):
    __path__ = []
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return Stub(self.__name__ + "." + name)
    def __call__(self, *a, **k):
        return Stub("stub")
    def __mro_entries__(self, bases):
        return (object,)
    def __or__(self, other):
        return self
    __ror__ = __or__
    def __getitem__(self, key):
        return self
    def __iter__(self):
        return iter(())
class Finder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, name, path, target=None):
        if name.split(".")[0] in STUBS:
            return importlib.machinery.ModuleSpec(name, self, is_package=True)
    def create_module(self, spec):
        return Stub(spec.name)
    def exec_module(self, module):
        pass
sys.meta_path.insert(0, Finder())
_version = importlib.metadata.version
importlib.metadata.version = lambda name: "0.15.3" if name == "openmc" else _version(name)

# the drop-in switch: openmc/lib/__init__.py opens this library
_CDLL = ctypes.CDLL
def CDLL(name, *a, **k):
    if str(name).endswith("libopenmc.so"):
        name = lib_path
    return _CDLL(name, *a, **k)
ctypes.CDLL = CDLL

sys.path.insert(0, ref)
import openmc.lib as ol
assert ol.__file__.startswith(ref)
ol.init([model_dir], output=False)
out = {
    "event_based": bool(ol.settings.event_based),
    "particles": int(ol.settings.particles),
    "run_mode": ol.settings.run_mode,
    "cells": sorted(int(k) for k in ol.cells.keys()),
    "materials": sorted(int(k) for k in ol.materials.keys()),
    "tallies": sorted(int(k) for k in ol.tallies.keys()),
    "meshes": sorted(int(k) for k in ol.meshes.keys()),
    "nuclides": sorted(ol.materials[sorted(ol.materials.keys())[0]].nuclides),
    "mesh_dimension": [int(v) for v in ol.meshes[sorted(ol.meshes.keys())[0]].dimension],
    "bbox": [list(map(float, v)) for v in ol.global_bounding_box()],
    "is_initialized": bool(ol.is_initialized),
}
t = ol.tallies[out["tallies"][0]]
out["tally"] = {"estimator": t.estimator, "scores": list(t.scores), "n_realizations": int(t.num_realizations),
                "filters": [type(f).__name__ for f in t.filters]}
ef = [f for f in t.filters if type(f).__name__ == "EnergyFilter"][0]
out["energy_bins"] = [float(ef.bins[0]), float(ef.bins[-1]), len(ef.bins) - 1]
mf = [f for f in t.filters if type(f).__name__ == "MeshFilter"][0]
out["mesh_filter_mesh"] = int(mf.mesh.id)
c = ol.cells[out["cells"][0]]
out["cell0_fill"] = type(c.fill).__name__
# no GPU in this container: the transport path fails loudly through the
# reference's own error mapping (there is no CPU fallback)
try:
    ol.simulation_init()
    out["simulation_init"] = "ran"
except ol.exc.OpenMCError as e:
    out["simulation_init"] = type(e).__name__ + ": " + str(e)[:80]
ol.hard_reset()
ol.finalize()
out["is_initialized_after"] = bool(ol.is_initialized)
print(json.dumps(out))
'''


def test_reference_openmc_lib_drives_this_library(built, tmp_path):
    if not (REF / "openmc" / "lib" / "__init__.py").exists():
        pytest.skip("reference tree not present")
    from openmc_gb300 import configs, lib
    m, d = configs.lattice17(tmp_path, particles=1000, batches=3, n_points=300, mesh_dim=(17, 17, 5), n_ebins=4)
    m.export_to_model_xml(d / "model.xml")
    r = subprocess.run([sys.executable, "-c", SCRIPT, str(REF), lib.loaded_library(), str(d)],
                       capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["is_initialized"] and not out["is_initialized_after"]
    assert out["particles"] == 1000 and out["run_mode"] == "fixed source"
    assert out["event_based"] is True
    assert len(out["cells"]) == 7 and len(out["meshes"]) == 1
    assert out["materials"] == sorted(x.id for x in m.materials)
    assert out["tallies"] == sorted(t.id for t in m.tallies)
    assert out["nuclides"] == sorted(["Hv235", "Hv238", "Ox16", "Hv240"])
    assert out["mesh_dimension"] == [17, 17, 5]
    assert out["tally"] == {"estimator": "tracklength", "scores": ["flux"], "n_realizations": 0,
                            "filters": ["MeshFilter", "EnergyFilter"]}
    assert out["energy_bins"][2] == 4 and out["mesh_filter_mesh"] == out["meshes"][0]
    import torch
    if not torch.cuda.is_available():
        assert out["simulation_init"].split(":")[0].endswith("Error"), out["simulation_init"]
    assert abs(out["bbox"][0][0] + 10.71) < 1e-9 and abs(out["bbox"][1][2] - 100.0) < 1e-9
