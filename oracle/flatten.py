"""Oracle test infrastructure: read ``model.xml`` + nuclide files into flat arrays.

This is the CPU oracle's own model reader.  It is deliberately independent of
the C++ XML reader inside the product library: the oracle and the product
parse the same ``model.xml`` with separate code, so a parsing mistake on
either side shows up as a parity failure.

It follows the meaning the reference gives each element:
materials ``src/material.cpp`` (atom fractions, density), surfaces
``src/surface.cpp`` (type + coeffs + boundary), cells ``src/cell.cpp``
(universe, fill, material, region, translation), rectangular lattices
``src/lattice.cpp:160-230`` (universes listed top row first), meshes
``src/mesh.cpp`` (dimension, lower_left, upper_right/width), filters
``src/tallies/filter_*.cpp``, settings ``src/settings.cpp`` and weight windows
``src/weight_windows.cpp``.

Output: a dict of numpy arrays (int64 or float64) serialised by
:func:`to_blob` into the byte format read by ``oracle.cpp``.
"""
from __future__ import annotations

import os
import struct
from pathlib import Path
from xml.etree import ElementTree as ET

import numpy as np

INFTY = float.fromhex('0x1.fffffffffffffp+1023')  # include/openmc/constants.h INFTY (largest double)


def _read_library(xml_path):
    """name -> nuclide file path from a cross_sections.xml (OpenMC schema)."""
    xml_path = Path(xml_path)
    out = {}
    for lib in ET.parse(xml_path).getroot().iter("library"):
        p = Path(lib.get("path"))
        if not p.is_absolute():
            p = xml_path.parent / p
        for m in lib.get("materials").split():
            out[m] = p
    return out


def _read_nuclide(path):
    """Read the native nuclide container (see openmc_gb300/data.py header):
    returns (awr, kT, energy, {mt: (threshold_idx, xs)}, fission) with
    fission None or (nu0, nu1, spectrum, p0, p1, u)."""
    buf = Path(path).read_bytes()
    if buf[:8] != b"OMCGBNUC":
        raise ValueError(f"{path}: not a nuclide file")
    (version,) = struct.unpack_from("<I", buf, 8)
    off = 12
    (nlen,) = struct.unpack_from("<I", buf, off); off += 4 + nlen
    _A, awr, kT = struct.unpack_from("<3d", buf, off); off += 24
    n, nrx = struct.unpack_from("<II", buf, off); off += 8
    energy = np.frombuffer(buf, "<f8", n, off).copy(); off += 8 * n
    rx = {}
    for _ in range(nrx):
        mt, thr, m = struct.unpack_from("<III", buf, off); off += 12
        rx[mt] = (thr, np.frombuffer(buf, "<f8", m, off).copy()); off += 8 * m
    fission = None
    if version >= 2:
        (flag,) = struct.unpack_from("<I", buf, off); off += 4
        if flag:
            nu0, nu1 = struct.unpack_from("<2d", buf, off); off += 16
            (spec,) = struct.unpack_from("<I", buf, off); off += 4
            p0, p1, u = struct.unpack_from("<3d", buf, off); off += 24
            fission = (nu0, nu1, spec, p0, p1, u)
    return awr, kT, energy, rx, fission


SURF_TYPES = {"x-plane": 0, "y-plane": 1, "z-plane": 2, "x-cylinder": 3,
              "y-cylinder": 4, "z-cylinder": 5, "sphere": 6}
BC = {"transmission": 0, "vacuum": 1, "reflective": 2}
# Region operator tokens: include/openmc/cell.h:31-35
OP_LEFT_PAREN = 2**31 - 1
OP_RIGHT_PAREN = 2**31 - 2
OP_COMPLEMENT = 2**31 - 3
OP_INTERSECTION = 2**31 - 4
OP_UNION = 2**31 - 5
SCORES = {"flux": 0, "total": 1, "absorption": 2}


def _floats(text):
    return [float(v) for v in text.split()]


def _ints(text):
    return [int(v) for v in text.split()]


def _get(node, name, default=None):
    """Attribute or child-element text, as the reference's get_node_value."""
    if name in node.attrib:
        return node.attrib[name]
    ch = node.find(name)
    if ch is not None and ch.text is not None:
        return ch.text.strip()
    return default


def _region_tokens(spec, surf_index):
    """Tokenise a region string to the reference's infix token list.

    Returns (tokens, simple).  Simple regions keep only surface tokens
    (``src/cell.cpp:556-683``).  For regions with unions the tokens are
    converted to postfix here (the oracle evaluates postfix; the truth value
    equals the reference's infix scan).
    """
    toks = []
    i = 0
    while i < len(spec):
        ch = spec[i]
        if ch == "(":
            toks.append(OP_LEFT_PAREN); i += 1
        elif ch == ")":
            toks.append(OP_RIGHT_PAREN); i += 1
        elif ch == "|":
            toks.append(OP_UNION); i += 1
        elif ch == "~":
            toks.append(OP_COMPLEMENT); i += 1
        elif ch in "+-" or ch.isdigit():
            j = i + 1
            while j < len(spec) and spec[j].isdigit():
                j += 1
            toks.append(int(spec[i:j])); i = j
        elif ch.isspace():
            i += 1
        else:
            raise ValueError(f"invalid region character {ch!r}")
    # implicit intersections
    out = []
    for k, t in enumerate(toks):
        out.append(t)
        if k + 1 < len(toks):
            left = t < OP_UNION or t == OP_RIGHT_PAREN
            nxt = toks[k + 1]
            right = nxt < OP_UNION or nxt in (OP_LEFT_PAREN, OP_COMPLEMENT)
            if left and right:
                out.append(OP_INTERSECTION)
    # surface ids -> signed index+1
    conv = []
    for t in out:
        if t < OP_UNION:
            idx = surf_index[abs(t)] + 1
            conv.append(idx if t > 0 else -idx)
        else:
            conv.append(t)
    simple = OP_UNION not in conv and OP_COMPLEMENT not in conv
    if simple:
        return [t for t in conv if t < OP_UNION], True
    # shunting-yard to postfix; precedence: complement > intersection > union
    prec = {OP_COMPLEMENT: 3, OP_INTERSECTION: 2, OP_UNION: 1}
    post, stack = [], []
    for t in conv:
        if t < OP_UNION:
            post.append(t)
        elif t == OP_LEFT_PAREN:
            stack.append(t)
        elif t == OP_RIGHT_PAREN:
            while stack[-1] != OP_LEFT_PAREN:
                post.append(stack.pop())
            stack.pop()
            if stack and stack[-1] == OP_COMPLEMENT:
                post.append(stack.pop())
        elif t == OP_COMPLEMENT:
            stack.append(t)
        else:
            while stack and stack[-1] != OP_LEFT_PAREN and prec[stack[-1]] >= prec[t]:
                post.append(stack.pop())
            stack.append(t)
    while stack:
        post.append(stack.pop())
    return post, False


def load_model(model_xml, cross_sections=None):
    """Parse a model.xml into flat arrays for the oracle."""
    model_xml = Path(model_xml)
    root = ET.parse(model_xml).getroot()
    base = model_xml.parent
    mats_el = root.find("materials")
    geom_el = root.find("geometry")
    set_el = root.find("settings")
    tal_el = root.find("tallies")

    # ---- cross sections library
    xs_path = cross_sections
    if xs_path is None and mats_el.find("cross_sections") is not None:
        xs_path = mats_el.find("cross_sections").text.strip()
    if xs_path is None:
        xs_path = os.environ.get("OPENMC_CROSS_SECTIONS")
    xs_path = Path(xs_path)
    if not xs_path.is_absolute():
        xs_path = base / xs_path
    library = _read_library(xs_path)

    # ---- materials
    mat_ids, nuc_names = [], []
    mat_off, mat_nuc, mat_ao, mat_density = [0], [], [], []
    for m in mats_el.findall("material"):
        mat_ids.append(int(m.get("id")))
        d = m.find("density")
        units = d.get("units")
        for n in m.findall("nuclide"):
            name = n.get("name")
            if name not in nuc_names:
                nuc_names.append(name)
            mat_nuc.append(nuc_names.index(name))
            mat_ao.append(float(n.get("ao")))
        mat_off.append(len(mat_nuc))
        if units == "sum":
            mat_density.append(float(sum(mat_ao[mat_off[-2]:])))
        elif units == "atom/b-cm":
            mat_density.append(float(d.get("value")))
        else:
            raise ValueError(f"unsupported density units {units}")
    mat_index = {mid: k for k, mid in enumerate(mat_ids)}

    nuc_off, energy, elastic, capture, awr, kT = [0], [], [], [], [], []
    fission_xs, fis_i, fis_d = [], [], []
    for name in nuc_names:
        n_awr, n_kT, n_energy, rx, fis = _read_nuclide(library[name])
        thr_el, el = rx[2]
        thr_c, cap = rx[102]
        if thr_el != 0 or thr_c != 0:
            raise ValueError("threshold reactions are not supported")
        energy.append(n_energy); elastic.append(el); capture.append(cap)
        awr.append(n_awr); kT.append(n_kT)
        nuc_off.append(nuc_off[-1] + len(n_energy))
        if fis is not None and 18 in rx:
            fission_xs.append(rx[18][1])
            fis_i.extend([1, fis[2]])
            fis_d.extend([fis[0], fis[1], fis[3], fis[4], fis[5]])
        else:
            fission_xs.append(np.zeros(len(n_energy)))
            fis_i.extend([0, 0])
            fis_d.extend([0.0] * 5)

    # ---- geometry
    surfs = geom_el.findall("surface")
    surf_index = {int(s.get("id")): k for k, s in enumerate(surfs)}
    surf_type, surf_coeffs, surf_bc, surf_id = [], [], [], []
    for s in surfs:
        surf_id.append(int(s.get("id")))
        surf_type.append(SURF_TYPES[s.get("type")])
        c = _floats(s.get("coeffs"))
        surf_coeffs.extend(c + [0.0] * (4 - len(c)))
        surf_bc.append(BC[s.get("boundary", "transmission")])

    cells = geom_el.findall("cell")
    lats = geom_el.findall("lattice")
    univ_ids = []
    for c in cells:
        u = int(c.get("universe", 0))
        if u not in univ_ids:
            univ_ids.append(u)
    univ_index = {u: k for k, u in enumerate(univ_ids)}
    lat_index = {int(l.get("id")): k for k, l in enumerate(lats)}

    cell_id, cell_univ, cell_ftype, cell_fill = [], [], [], []
    cell_tok_off, cell_tok, cell_simple, cell_trans = [0], [], [], []
    filled = set()
    for c in cells:
        cell_id.append(int(c.get("id")))
        cell_univ.append(univ_index[int(c.get("universe", 0))])
        if c.get("fill") is not None:
            f = int(c.get("fill"))
            filled.add(f)
            if f in lat_index:
                cell_ftype.append(2); cell_fill.append(lat_index[f])
            else:
                cell_ftype.append(1); cell_fill.append(univ_index[f])
        else:
            mat = c.get("material")
            cell_ftype.append(0)
            cell_fill.append(-1 if mat == "void" else mat_index[int(mat)])
        toks, simple = _region_tokens(c.get("region", ""), surf_index)
        cell_tok.extend(toks); cell_tok_off.append(len(cell_tok))
        cell_simple.append(1 if simple else 0)
        t = c.get("translation")
        cell_trans.extend(_floats(t) if t else [0.0, 0.0, 0.0])

    univ_cell_off, univ_cells = [0], []
    for u in range(len(univ_ids)):
        univ_cells.extend(k for k, cu in enumerate(cell_univ) if cu == u)
        univ_cell_off.append(len(univ_cells))

    lat_n, lat_ll, lat_pitch, lat_is3d, lat_outer = [], [], [], [], []
    lat_univ_off, lat_univ = [0], []
    for l in lats:
        dims = _ints(_get(l, "dimension"))
        is3d = len(dims) == 3
        n = dims + [1] * (3 - len(dims))
        ll = _floats(_get(l, "lower_left"))
        pitch = _floats(_get(l, "pitch"))
        words = _ints(_get(l, "universes"))
        for u in words:
            filled.add(u)
        flat = [0] * (n[0] * n[1] * n[2])
        for iz in range(n[2]):
            for iy in range(n[1] - 1, -1, -1):
                for ix in range(n[0]):
                    i1 = n[0] * n[1] * iz + n[0] * (n[1] - iy - 1) + ix
                    i2 = n[0] * n[1] * iz + n[0] * iy + ix
                    flat[i1] = univ_index[words[i2]]
        outer = _get(l, "outer")
        if outer is not None:
            filled.add(int(outer))
        lat_n.extend(n); lat_ll.extend(ll + [0.0] * (3 - len(ll)))
        lat_pitch.extend(pitch + [0.0] * (3 - len(pitch)))
        lat_is3d.append(1 if is3d else 0)
        lat_outer.append(univ_index[int(outer)] if outer is not None else -1)
        lat_univ.extend(flat); lat_univ_off.append(len(lat_univ))
    roots = [u for u in univ_ids if u not in filled]
    if len(roots) != 1:
        raise ValueError(f"could not identify the root universe: {roots}")
    root_univ = univ_index[roots[0]]

    # ---- meshes (tallies and settings)
    meshes = {}
    for el in list(set_el.findall("mesh")) + (list(tal_el.findall("mesh")) if tal_el is not None else []):
        if int(el.get("id")) in meshes:
            raise ValueError(f"Two or more meshes use the same unique ID: {el.get('id')}")
        dim = _ints(_get(el, "dimension"))
        ll = _floats(_get(el, "lower_left"))
        ur = _get(el, "upper_right")
        width = _get(el, "width")
        meshes[int(el.get("id"))] = (dim, ll, _floats(ur) if ur else None,
                                     _floats(width) if width else None)
    mesh_ids = sorted(meshes)
    mesh_index = {m: k for k, m in enumerate(mesh_ids)}
    mesh_dim, mesh_ll, mesh_ur, mesh_width, mesh_ndim = [], [], [], [], []
    for m in mesh_ids:
        dim, ll, ur, width = meshes[m]
        nd = len(dim)
        mesh_ndim.append(nd)
        mesh_dim.extend(dim + [1] * (3 - nd))
        mesh_ll.extend(ll + [0.0] * (3 - nd))
        if width is not None:
            # upper_right = lower_left + shape * width (src/mesh.cpp:1216)
            mesh_width.extend(width + [1.0] * (3 - nd))
            mesh_ur.extend([ll[i] + dim[i] * width[i] for i in range(nd)] + [1.0] * (3 - nd))
        else:
            mesh_ur.extend(ur + [1.0] * (3 - nd))
            mesh_width.extend([(ur[i] - ll[i]) / dim[i] for i in range(nd)] + [1.0] * (3 - nd))

    # ---- tallies
    filt_type, filt_mesh, filt_nbins, filt_eoff, filt_e = [], [], [], [0], []
    filt_ioff, filt_ids = [0], []
    tal_id, tal_filt_off, tal_filt, tal_score_off, tal_score, tal_est = [], [0], [], [0], [], []
    cell_index = {int(c.get("id")): k for k, c in enumerate(cells)}
    if tal_el is not None:
        filters = tal_el.findall("filter")
        filt_index = {int(f.get("id")): k for k, f in enumerate(filters)}
        for f in filters:
            t = f.get("type")
            bins = _get(f, "bins")
            if t == "mesh":
                filt_type.append(0)
                mi = mesh_index[int(bins)]
                filt_mesh.append(mi)
                filt_nbins.append(int(np.prod(mesh_dim[3 * mi:3 * mi + 3])))
            elif t == "energy":
                e = _floats(bins)
                filt_type.append(1); filt_mesh.append(-1)
                filt_nbins.append(len(e) - 1)
                filt_e.extend(e)
            elif t == "particle":
                if bins.split() != ["neutron"]:
                    raise ValueError("only neutron particle filters are supported")
                filt_type.append(2); filt_mesh.append(-1); filt_nbins.append(1)
            elif t in ("cell", "material"):
                # src/tallies/filter_cell.cpp, filter_material.cpp: bins are ids
                index = cell_index if t == "cell" else mat_index
                ids = [index[i] for i in _ints(bins)]
                filt_type.append(3 if t == "cell" else 4); filt_mesh.append(-1)
                filt_nbins.append(len(ids))
                filt_ids.extend(ids)
            else:
                raise ValueError(f"unsupported filter type {t}")
            filt_eoff.append(len(filt_e))
            filt_ioff.append(len(filt_ids))
        for t in tal_el.findall("tally"):
            tal_id.append(int(t.get("id")))
            fl = _get(t, "filters")
            for fid in (_ints(fl) if fl else []):
                tal_filt.append(filt_index[fid])
            tal_filt_off.append(len(tal_filt))
            est = _get(t, "estimator", "tracklength")
            if est not in ("tracklength", "collision"):
                raise ValueError("only track-length and collision estimators are supported")
            tal_est.append(0 if est == "tracklength" else 1)
            for s in _get(t, "scores").split():
                tal_score.append(SCORES[s])
            tal_score_off.append(len(tal_score))

    # ---- settings
    particles = int(_get(set_el, "particles"))
    batches = int(_get(set_el, "batches"))
    inactive = int(_get(set_el, "inactive", 0))
    run_mode = (_get(set_el, "run_mode", "fixed source") or "fixed source").strip()
    if run_mode not in ("fixed source", "eigenvalue"):
        raise ValueError(f"run mode {run_mode} is not supported")
    gen_per_batch = int(_get(set_el, "generations_per_batch", 1))
    seed = int(_get(set_el, "seed", 1))
    log_grid_bins = int(_get(set_el, "log_grid_bins", 8000))
    max_split_hist = int(_get(set_el, "max_history_splits", 10_000_000))
    event_based = (_get(set_el, "event_based", "false").lower() == "true")
    e_cut = 0.0
    co = set_el.find("cutoff")
    if co is not None and _get(co, "energy_neutron") is not None:
        e_cut = float(_get(co, "energy_neutron"))
    # src/settings.cpp:723-724 time_cutoff[neutron] (INFTY: none)
    t_cut = INFTY
    if co is not None and _get(co, "time_neutron") is not None:
        t_cut = float(_get(co, "time_neutron"))

    # ---- source (one independent source)
    srcs = set_el.findall("source")
    if len(srcs) != 1:
        raise ValueError("exactly one source is supported")
    src = srcs[0]
    space = src.find("space")
    sp_type = {"point": 0, "box": 1}[space.get("type")]
    sp_par = _floats(_get(space, "parameters"))
    angle = src.find("angle")
    an_type = {"isotropic": 0, "monodirectional": 1}[angle.get("type", "isotropic")]
    an_ref = _floats(angle.get("reference_uvw", "1 0 0"))
    energy_el = src.find("energy")
    en_type = {"discrete": 0, "maxwell": 1}[energy_el.get("type")]
    en_par = _floats(_get(energy_el, "parameters"))
    strength = float(src.get("strength", 1.0))
    dom_type, dom_ids = -1, []
    cons = src.find("constraints")
    if cons is None:
        cons = src
    if _get(cons, "domain_type") is not None:
        dom_type = {"cell": 0, "material": 1, "universe": 2}[_get(cons, "domain_type")]
        dom_ids = _ints(_get(cons, "domain_ids"))

    # ---- weight windows (first set only)
    ww_on = 0
    ww_i, ww_d, ww_e, ww_lower, ww_upper = [-1, 0, 10], [3.0, 1.0, 1.0e-38], [], [], []
    wws = set_el.findall("weight_windows")
    if wws:
        w = wws[0]
        ww_on = 1
        if _get(set_el, "weight_windows_on") is not None:
            ww_on = 1 if _get(set_el, "weight_windows_on").lower() == "true" else 0
        mi = mesh_index[int(_get(w, "mesh"))]
        ww_e = _floats(_get(w, "energy_bounds"))
        ww_lower = _floats(_get(w, "lower_ww_bounds"))
        ww_upper = _floats(_get(w, "upper_ww_bounds"))
        n_ww = (len(ww_e) - 1) * int(np.prod(mesh_dim[3 * mi:3 * mi + 3]))
        if len(ww_lower) != n_ww or len(ww_upper) != n_ww:
            raise ValueError("weight-window bounds have the wrong size")
        mlb = _get(w, "max_lower_bound_ratio")
        ww_i = [mi, 1, int(_get(w, "max_split", 10))]
        ww_d = [float(_get(w, "survival_ratio", 3.0)),
                float(mlb) if mlb is not None else 1.0,
                float(_get(w, "weight_cutoff", 1.0e-38))]

    I = lambda v: np.asarray(v, dtype=np.int64)
    D = lambda v: np.asarray(v, dtype=np.float64)
    return {
        "settings_i": I([particles, batches, inactive, seed, log_grid_bins,
                         max_split_hist, 1 if event_based else 0, ww_on]),
        "settings_d": D([e_cut, t_cut]),
        "nuc_off": I(nuc_off), "nuc_awr": D(awr), "nuc_kT": D(kT),
        "nuc_energy": D(np.concatenate(energy)),
        "nuc_elastic": D(np.concatenate(elastic)),
        "nuc_capture": D(np.concatenate(capture)),
        "nuc_fission": D(np.concatenate(fission_xs)),
        "nuc_fis_i": I(fis_i), "nuc_fis_d": D(fis_d),
        "eig_i": I([1 if run_mode == "eigenvalue" else 0, gen_per_batch]), "eig_d": D([1.0]),
        "mat_id": I(mat_ids), "mat_off": I(mat_off), "mat_nuc": I(mat_nuc),
        "mat_ao": D(mat_ao), "mat_density": D(mat_density),
        "surf_id": I(surf_id), "surf_type": I(surf_type),
        "surf_coeffs": D(surf_coeffs), "surf_bc": I(surf_bc),
        "cell_id": I(cell_id), "cell_univ": I(cell_univ),
        "cell_ftype": I(cell_ftype), "cell_fill": I(cell_fill),
        "cell_tok_off": I(cell_tok_off), "cell_tok": I(cell_tok),
        "cell_simple": I(cell_simple), "cell_trans": D(cell_trans),
        "univ_cell_off": I(univ_cell_off), "univ_cells": I(univ_cells),
        "root_univ": I([root_univ]),
        "lat_n": I(lat_n), "lat_ll": D(lat_ll), "lat_pitch": D(lat_pitch),
        "lat_is3d": I(lat_is3d), "lat_outer": I(lat_outer),
        "lat_univ_off": I(lat_univ_off), "lat_univ": I(lat_univ),
        "mesh_ndim": I(mesh_ndim), "mesh_dim": I(mesh_dim), "mesh_ll": D(mesh_ll),
        "mesh_ur": D(mesh_ur), "mesh_width": D(mesh_width),
        "filt_type": I(filt_type), "filt_mesh": I(filt_mesh),
        "filt_nbins": I(filt_nbins), "filt_eoff": I(filt_eoff), "filt_e": D(filt_e),
        "filt_ioff": I(filt_ioff), "filt_ids": I(filt_ids),
        "tal_id": I(tal_id), "tal_filt_off": I(tal_filt_off), "tal_filt": I(tal_filt),
        "tal_score_off": I(tal_score_off), "tal_score": I(tal_score), "tal_est": I(tal_est),
        "src_i": I([sp_type, an_type, en_type, dom_type]),
        "src_space": D(sp_par), "src_uref": D(an_ref), "src_energy": D(en_par),
        "src_strength": D([strength]), "src_dom_ids": I(dom_ids),
        "ww_i": I(ww_i), "ww_d": D(ww_d), "ww_e": D(ww_e),
        "ww_lower": D(ww_lower), "ww_upper": D(ww_upper),
    }


def to_blob(arrays: dict) -> bytes:
    """Serialise named arrays: b'OMCFLAT1', u32 count, then per array
    u8 name length, name, u8 kind ('i' int64 / 'd' float64), u64 n, data."""
    out = [b"OMCFLAT1", struct.pack("<I", len(arrays))]
    for name, arr in arrays.items():
        nb = name.encode()
        kind = b"i" if arr.dtype == np.int64 else b"d"
        out.append(struct.pack("<B", len(nb)) + nb + kind + struct.pack("<Q", arr.size))
        out.append(np.ascontiguousarray(arr).tobytes())
    return b"".join(out)
