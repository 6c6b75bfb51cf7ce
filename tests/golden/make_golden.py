"""Generate the golden fixtures that pin the oracle to the reference.

Run in a container where the reference tree is mounted (the argument, else
OPENMC_REF_ROOT, else /root/reference) after ``oracle/build_ref.sh`` has compiled the reference's
src/random_lcg.cpp into oracle/_ref/:

    python tests/golden/make_golden.py [reference_root]

Writes
  test_math_golden.json  known answers parsed from the reference's
                         tests/cpp_unit_tests/test_math.cpp (rotate_angle,
                         maxwell_spectrum, watt_spectrum with seed 1)
  rng_golden.json        prn() sequences, future_seed() skips and init_seed()
                         values produced by the reference's own random_lcg.cpp
"""
import json
import os
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))


def parse_test_math(ref_root: Path):
    src = (ref_root / "tests/cpp_unit_tests/test_math.cpp").read_text()
    out = {}
    m = re.search(r'TEST_CASE\("Test maxwell_spectrum"\).*?ref_val = ([0-9.eE+-]+);.*?double T = ([0-9.]+);'
                  r'.*?prn_seed = (\d+);', src, re.S)
    out["maxwell_spectrum"] = {"T": float(m.group(2)), "seed": int(m.group(3)), "value": float(m.group(1))}
    m = re.search(r'TEST_CASE\("Test watt_spectrum"\).*?ref_val = ([0-9.eE+-]+);.*?double a = ([0-9.]+);'
                  r'.*?double b = ([0-9.]+);.*?prn_seed = (\d+);', src, re.S)
    out["watt_spectrum"] = {"a": float(m.group(2)), "b": float(m.group(3)), "seed": int(m.group(4)),
                            "value": float(m.group(1))}
    m = re.search(r'SECTION\("Test rotate_angle no phi"\).*?ref_uvw = \{\s*([^}]*)\};.*?double mu = ([0-9.]+);'
                  r'.*?prn_seed = (\d+);', src, re.S)
    vals = [float(v) for v in m.group(1).replace("\n", " ").split(",")]
    out["rotate_angle_no_phi"] = {"uvw0": [1.0, 0.0, 0.0], "mu": float(m.group(2)), "seed": int(m.group(3)),
                                  "value": vals, "approx": True}
    m = re.search(r'SECTION\("Test rotate_angle mu is 0"\).*?ref_uvw \{([^}]*)\};', src, re.S)
    out["rotate_angle_mu0_phi0"] = {"uvw0": [1.0, 0.0, 0.0], "mu": 0.0, "phi": 0.0,
                                    "value": [float(v) for v in m.group(1).split(",")], "approx": True}
    m = re.search(r'SECTION\("Test rotate_angle mu is 1"\).*?ref_uvw = \{([^}]*)\};', src, re.S)
    out["rotate_angle_mu1_phi0"] = {"uvw0": [1.0, 0.0, 0.0], "mu": 1.0, "phi": 0.0,
                                    "value": [float(v) for v in m.group(1).split(",")], "approx": True}
    out["source"] = "tests/cpp_unit_tests/test_math.cpp:204-276"
    return out


def rng_vectors():
    import ctypes as C
    import oracle
    ref = oracle.ref_lib()
    if ref is None:
        raise SystemExit("oracle/_ref/librandom_lcg_ref.so missing: run oracle/build_ref.sh first")
    seqs = {}
    for seed in (1, 12345, 2**63 + 17):
        s = C.c_uint64(seed)
        vals = []
        for _ in range(16):
            vals.append(ref.ref_prn(C.byref(s)).hex())
        seqs[str(seed)] = {"prn_hex": vals, "final_state": s.value}
    skips = []
    for n, seed in [(0, 1), (1, 1), (152917, 1), (152917 * 10**7, 2), (2**40 + 3, 99)]:
        skips.append({"n": n, "seed": seed, "value": ref.ref_future_seed(n, seed)})
    inits = []
    for id_, off, master, stride in [(1, 0, 1, 152917), (1, 1, 1, 152917), (10**7, 0, 1, 152917),
                                     (123456789, 1, 7, 152917), (5, 0, 1, 1000)]:
        inits.append({"id": id_, "offset": off, "master": master, "stride": stride,
                      "value": ref.ref_init_seed(id_, off, master, stride)})
    return {"prn": seqs, "future_seed": skips, "init_seed": inits,
            "source": "reference src/random_lcg.cpp compiled by oracle/build_ref.sh"}


if __name__ == "__main__":
    ref_root = Path(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("OPENMC_REF_ROOT", "/root/reference"))
    (HERE / "test_math_golden.json").write_text(json.dumps(parse_test_math(ref_root), indent=1))
    (HERE / "rng_golden.json").write_text(json.dumps(rng_vectors(), indent=1))
    print("wrote", HERE / "test_math_golden.json", HERE / "rng_golden.json")
