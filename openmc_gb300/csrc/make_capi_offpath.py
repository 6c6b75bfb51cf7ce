"""Writes capi_offpath.cpp: the openmc.lib entry points outside the
event-based fixed-source path, so that the reference's Python bindings,
which declare argument types for every function they use at import
(openmc/lib/*.py), load this library.  Each returns OPENMC_E_UNASSIGNED with
a message naming the function (void functions only set the message; bool
functions return false).

The functions written are those the reference's bindings name (openmc_*
entry points and the few others they bind, such as the Zernike helpers of
openmc/lib/math.py) and no other source file of this directory defines; their prototypes are read from the
reference's include/openmc headers and, for the few declared only there,
from the extern "C" definitions in its src/ files.

    python make_capi_offpath.py <reference checkout> > capi_offpath.cpp
    python make_capi_offpath.py <reference checkout> --header > ../../include/openmc_gb300_offpath.h
"""
import glob
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def _strip_comments(text):
    text = re.sub(r'//[^\n]*', '', text)
    return re.sub(r'/\*.*?\*/', '', text, flags=re.S)


def bound_names(ref):
    names = set()
    for f in glob.glob(str(ref / "openmc" / "lib" / "*.py")):
        names |= set(re.findall(r'_dll\.([A-Za-z]\w*)', Path(f).read_text()))
    return names


def defined_here():
    names = set()
    for f in list(HERE.glob("*.cpp")) + list(HERE.glob("*.cu")):
        if f.name == "capi_offpath.cpp":
            continue
        names |= set(re.findall(r'^(?:extern "C" )?[\w\s\*]*?\b([A-Za-z]\w*)\s*\([^;]*?\)\s*\{',
                                _strip_comments(f.read_text()), flags=re.M))
    return names


def prototypes(ref, names):
    headers = "".join(Path(h).read_text() + "\n" for h in
                      sorted(glob.glob(str(ref / "include" / "openmc" / "**" / "*.h"), recursive=True)))
    sources = "".join(Path(s).read_text() + "\n" for s in
                      sorted(glob.glob(str(ref / "src" / "**" / "*.cpp"), recursive=True)))
    headers, sources = _strip_comments(headers), _strip_comments(sources)
    out = {}
    for n in sorted(names):
        m = re.search(r'(?:extern\s+"C"\s+)?([A-Za-z_][\w\s\*]*?)\b' + n + r'\s*\(([^;{]*?)\)\s*;', headers, re.S)
        if not m:
            m = re.search(r'\n\s*(?:extern\s+"C"\s+)?([A-Za-z_][\w\s\*]*?)\b' + n + r'\s*\(([^;{]*?)\)\s*\{',
                          sources, re.S)
        if not m:
            raise SystemExit(f"no prototype found for {n}")
        ret = m.group(1).split()[-1]
        params = re.sub(r'\s*=\s*[^,]+', '', " ".join(m.group(2).split()))  # C++ default arguments
        out[n] = (ret, params)
    return out


def header(decl):
    out = ['/* Generated by openmc_gb300/csrc/make_capi_offpath.py: the openmc.lib entry',
           ' * points outside the event-based fixed-source path that this library',
           ' * exports only so that the reference\'s Python bindings (openmc/lib/*.py)',
           ' * load it.  Prototypes as in the reference\'s include/openmc/capi.h (or its',
           ' * src/ definitions); every call returns OPENMC_E_UNASSIGNED with a message',
           ' * in openmc_err_msg (void functions only set the message, bool functions',
           ' * return false). */',
           '#ifndef OPENMC_GB300_OFFPATH_H', '#define OPENMC_GB300_OFFPATH_H', '',
           '#include <stdbool.h>', '#include <stddef.h>', '#include <stdint.h>', '',
           '#ifdef __cplusplus', 'extern "C" {', '#endif', '',
           'typedef struct { double x, y, z; } openmc_gb300_position;  /* Position */', '']
    for name, (ret, params) in sorted(decl.items()):
        params = params.replace("Position", "openmc_gb300_position") or "void"
        out.append(f'{ret} {name}({params});')
    out += ['', '#ifdef __cplusplus', '}', '#endif', '#endif']
    return '\n'.join(out)


def main():
    ref = Path(sys.argv[1])
    decl = prototypes(ref, bound_names(ref) - defined_here())
    if "--header" in sys.argv[2:]:
        print(header(decl))
        return
    out = ['// Generated by make_capi_offpath.py: openmc.lib entry points outside the',
           '// event-based fixed-source transport path (model mutation, plotting,',
           '// volumes, depletion, CMFD, DAGMC, statepoints, source banks, other mesh and',
           '// filter types).  The reference binds every one of them at import',
           '// (openmc/lib/*.py); here each reports that it is not available.',
           '#include <cstddef>', '#include <cstdint>', '#include <cstdio>', '',
           'extern "C" {', 'extern int OPENMC_E_UNASSIGNED;', 'extern char openmc_err_msg[256];', '}', '',
           'namespace {', 'struct Position {', '  double x, y, z;', '};', '',
           'int off_path(const char* name)', '{',
           '  std::snprintf(openmc_err_msg, 256, "%s is not available in the GB300 transport library "',
           '                "(outside the event-based fixed-source path).", name);',
           '  return OPENMC_E_UNASSIGNED;', '}', '}  // namespace', '', 'extern "C" {', '']
    for name, (ret, params) in sorted(decl.items()):
        out.append(f'{ret} {name}({params})')
        if ret == 'void':
            out += ['{', f'  off_path("{name}");', '}']
        elif ret == 'bool':
            out += ['{', f'  off_path("{name}");', '  return false;', '}']
        else:
            out.append(f'{{ return off_path("{name}"); }}')
        out.append('')
    out.append('}  // extern "C"')
    print('\n'.join(out))


if __name__ == '__main__':
    main()
