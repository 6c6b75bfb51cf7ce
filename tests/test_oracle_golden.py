"""The oracle pinned to the reference: the known answers of the reference's
tests/cpp_unit_tests/test_math.cpp and PRN/seed vectors produced by the
reference's own src/random_lcg.cpp (tests/golden/*.json)."""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def math_gold():
    return json.loads((GOLD / "test_math_golden.json").read_text())


@pytest.fixture(scope="module")
def rng_gold():
    return json.loads((GOLD / "rng_golden.json").read_text())


def test_maxwell_exact(math_gold):
    g = math_gold["maxwell_spectrum"]
    assert oracle.maxwell_spectrum(g["T"], g["seed"]) == g["value"]


def test_watt_exact(math_gold):
    g = math_gold["watt_spectrum"]
    assert oracle.watt_spectrum(g["a"], g["b"], g["seed"]) == g["value"]


def test_rotate_angle_no_phi(math_gold):
    g = math_gold["rotate_angle_no_phi"]
    u, _ = oracle.rotate_angle(g["uvw0"], g["mu"], None, g["seed"])
    assert np.allclose(u, g["value"], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("key", ["rotate_angle_mu0_phi0", "rotate_angle_mu1_phi0"])
def test_rotate_angle_fixed_phi(math_gold, key):
    g = math_gold[key]
    _, s = oracle.prn(1)
    u, _ = oracle.rotate_angle(g["uvw0"], g["mu"], g["phi"], s)
    assert np.allclose(u, g["value"], atol=1e-12)


def test_prn_sequences_bit_exact(rng_gold):
    for seed, d in rng_gold["prn"].items():
        s = int(seed)
        for hx in d["prn_hex"]:
            v, s = oracle.prn(s)
            assert v == float.fromhex(hx)
        assert s == d["final_state"]


def test_future_seed(rng_gold):
    for d in rng_gold["future_seed"]:
        assert oracle.future_seed(d["n"], d["seed"]) == d["value"]


def test_init_seed(rng_gold):
    for d in rng_gold["init_seed"]:
        assert oracle.init_seed(d["id"], d["offset"], d["master"], d["stride"]) == d["value"]


def test_against_compiled_reference_rng():
    """Direct comparison with the reference's random_lcg.cpp when it was
    compiled here (oracle/_ref is absent on machines without the tree)."""
    import ctypes as C
    ref = oracle.ref_lib()
    if ref is None:
        pytest.skip("reference random_lcg.cpp not compiled on this machine")
    rng = np.random.default_rng(3)
    for seed in rng.integers(0, 2**63, 50):
        s_ref = C.c_uint64(int(seed))
        s = int(seed)
        for _ in range(20):
            v, s = oracle.prn(s)
            assert v == ref.ref_prn(C.byref(s_ref))
        n = int(rng.integers(0, 2**62))
        assert oracle.future_seed(n, int(seed)) == ref.ref_future_seed(n, int(seed))


def test_against_compiled_reference_spectra():
    """The oracle's Maxwell and Watt fission spectra (the source energy and
    fission neutron samplers) against the reference's random_dist.cpp compiled
    here: the same values and the same seed advance, bit for bit."""
    import ctypes as C
    ref = oracle.ref_lib()
    if ref is None or not hasattr(ref, "ref_watt"):
        pytest.skip("reference random_dist.cpp not compiled on this machine")
    L = oracle.lib()
    rng = np.random.default_rng(11)
    for seed in rng.integers(0, 2**63, 200):
        for T in (2.0e4, 1.2895e6, 1.0e7):
            a, b = C.c_uint64(int(seed)), C.c_uint64(int(seed))
            for _ in range(25):
                assert L.oracle_maxwell_spectrum(T, C.byref(a)) == ref.ref_maxwell(T, C.byref(b))
            assert a.value == b.value
        for wa, wb in ((0.988e6, 2.249e-6), (1.0e6, 1.0e-6), (0.8e6, 4.0e-6)):
            a, b = C.c_uint64(int(seed)), C.c_uint64(int(seed))
            for _ in range(25):
                assert L.oracle_watt_spectrum(wa, wb, C.byref(a)) == ref.ref_watt(wa, wb, C.byref(b))
            assert a.value == b.value


def test_against_compiled_reference_grid_search():
    """The oracle's lower_bound_index (energy-grid and energy-filter search)
    against the reference's include/openmc/search.h compiled here: grids with
    repeated points (resonance and threshold duplicates), values on grid
    points, between them and at both ends."""
    import ctypes as C
    ref = oracle.ref_lib()
    if ref is None or not hasattr(ref, "ref_lower_bound_index"):
        pytest.skip("reference search.h not compiled on this machine")
    L = oracle.lib()
    rng = np.random.default_rng(5)
    for n in (2, 3, 17, 1000, 11303):
        g = np.sort(rng.uniform(1e-5, 2e7, n))
        g[rng.integers(1, n, max(1, n // 20))] = g[rng.integers(0, n - 1, max(1, n // 20))]
        g = np.sort(g)
        vals = np.concatenate([g, rng.uniform(g[0], g[-1], 2000), [g[0], g[-1]],
                               np.nextafter(g, np.inf)[:-1], np.nextafter(g, -np.inf)[1:]])
        p = g.ctypes.data_as(C.POINTER(C.c_double))
        for v in vals:
            assert L.oracle_lower_bound_index(p, n, float(v)) == ref.ref_lower_bound_index(p, n, float(v))
