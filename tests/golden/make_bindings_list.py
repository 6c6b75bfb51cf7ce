"""Writes openmc_lib_bindings.json: the C functions and exported globals the
reference's Python bindings (openmc/lib/*.py) resolve in the shared
library, read from a reference checkout.

    python make_bindings_list.py <reference checkout>
"""
import json
import re
import sys
from pathlib import Path


def main():
    lib = Path(sys.argv[1]) / "openmc" / "lib"
    funcs, globs = set(), set()
    for f in sorted(lib.glob("*.py")):
        text = f.read_text()
        funcs |= set(re.findall(r"_dll\.([A-Za-z]\w*)", text))
        globs |= set(re.findall(r"in_dll\(_dll,\s*['\"](\w+)['\"]\)", text))
        globs |= set(re.findall(r"_DLLGlobal\(\w+,\s*['\"](\w+)['\"]\)", text))
    out = Path(__file__).resolve().parent / "openmc_lib_bindings.json"
    out.write_text(json.dumps({"functions": sorted(funcs), "globals": sorted(globs)}, indent=1) + "\n")
    print(f"{len(funcs)} functions, {len(globs)} globals -> {out.name}")


if __name__ == "__main__":
    main()
