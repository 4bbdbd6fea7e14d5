"""Readers of the reference's input files: PAW-XML datasets (the JTH table's
`<paw_dataset>` format), the geometry file `cnt.ini` and the run parameters
`dim_paw.inp`.

`read_dataset` returns the tags the set-up chain of read_paw.f90 reads
(readpaw, read_paw.f90:1-67): the atom's charges (get_atom_charge,
read_paw.f90:652-678), the augmentation radius (get_rcut, :204-227), the
valence states with l and occupation (get_lstates_rcut, :403-427), the
radial grid values and derivatives (read_rr, :541-557), per state the
all-electron and pseudo partial waves and the projector (read_p_phi,
:482-539), the shape function's type and radius (get_comp, :68-110), the
Bloechl local ionic potential (read_vloc, :196-202), the pseudo valence
density the reference stores as its `ncoretilde` (read_ncoret,
:184-194), and what libpaw's dataset reader takes besides: the
all-electron and pseudo core densities and the kinetic-energy differences
K_ij that atompaw_dij0 starts D0 from (libpaw 2_m_paw_atom.F90:417).

Radial functions are returned as stored: the densities and the local
potential are the l = 0 components f_00 = sqrt(4 pi) f(r) (read_paw.f90
divides by sqrt(4 pi) or multiplies by Y_00), the partial waves and
projectors are the radial parts R(r) (not r R(r))."""
from __future__ import annotations

import xml.etree.ElementTree as ET

import numpy as np

_FUNCS = {
    "ae_core_density": "ae_core",
    "pseudo_core_density": "ps_core",
    "pseudo_valence_density": "ps_valence",
    "zero_potential": "zero_potential",
    "blochl_local_ionic_potential": "vloc_blochl",
}


def _floats(text):
    return np.array([float(v) for v in text.split()], dtype=np.float64)


def read_dataset(path):
    """Parses one PAW-XML dataset into a dict of numpy arrays and scalars
    (keys: symbol, Z, core, valence, rpaw, l, f, rc_state, e, ids, r, dr,
    shape_type, rcomp, phi, tphi, ptilde [nstates, nr], kij [nstates,
    nstates], and the radial functions of `_FUNCS`)."""
    root = ET.parse(path).getroot()
    if root.tag != "paw_dataset":
        raise ValueError(f"{path}: not a paw_dataset file (root tag {root.tag!r})")
    d = {}
    atom = root.find("atom")
    d["symbol"] = atom.get("symbol").strip()
    for k in ("Z", "core", "valence"):
        d[k] = float(atom.get(k))
    d["rpaw"] = float(root.find("paw_radius").get("rc"))
    states = root.find("valence_states").findall("state")
    d["ids"] = [s.get("id").strip() for s in states]
    d["l"] = np.array([int(s.get("l")) for s in states], np.int32)
    d["f"] = np.array([float(s.get("f")) if s.get("f") is not None else 0.0 for s in states])
    d["rc_state"] = np.array([float(s.get("rc")) for s in states])
    d["e"] = np.array([float(s.get("e")) for s in states])
    grids = root.findall("radial_grid")
    if len(grids) != 1:
        raise ValueError(f"{path}: {len(grids)} radial grids; one shared grid is supported")
    g = grids[0]
    istart, iend = int(g.get("istart")), int(g.get("iend"))
    r = _floats(g.find("values").text)
    dr = _floats(g.find("derivatives").text)
    if r.size != iend - istart + 1 or dr.size != r.size:
        raise ValueError(f"{path}: radial grid has {r.size} values for istart={istart}, iend={iend}")
    d["r"], d["dr"] = r, dr
    d["grid_eq"] = g.get("eq", "")
    sh = root.find("shape_function")
    d["shape_type"] = sh.get("type").strip()
    d["rcomp"] = float(sh.get("rc"))
    nr = r.size
    for tag, key in _FUNCS.items():
        el = root.find(tag)
        if el is None:
            d[key] = np.zeros(nr)
            continue
        v = _floats(el.text)
        if v.size != nr:
            raise ValueError(f"{path}: {tag} has {v.size} values, grid has {nr}")
        d[key] = v
    ns = len(states)
    for key, tag in (("phi", "ae_partial_wave"), ("tphi", "pseudo_partial_wave"), ("ptilde", "projector_function")):
        by_id = {e.get("state").strip(): _floats(e.text) for e in root.findall(tag)}
        rows = []
        for sid in d["ids"]:
            if sid not in by_id:
                raise ValueError(f"{path}: no {tag} for state {sid}")
            rows.append(by_id[sid])
        d[key] = np.stack(rows)
        if d[key].shape != (ns, nr):
            raise ValueError(f"{path}: {tag} arrays do not match the grid")
    k = _floats(root.find("kinetic_energy_differences").text)
    if k.size != ns * ns:
        raise ValueError(f"{path}: {k.size} kinetic-energy differences for {ns} states")
    d["kij"] = k.reshape(ns, ns)
    return d


def read_geometry(path):
    """`cnt.ini`: one atom per line, element symbol then x, y, z in Bohr
    (read_atominfo.f90).  Returns (symbols, coordinates [natom, 3])."""
    sym, xyz = [], []
    with open(path) as fh:
        for line in fh:
            t = line.split()
            if len(t) < 4:
                continue
            sym.append(t[0])
            xyz.append([float(v) for v in t[1:4]])
    return sym, np.array(xyz, dtype=np.float64)


def read_parameters(path):
    """`dim_paw.inp`: `key value` lines, `!` starts a comment.  Returns a
    dict of the values as strings (numbers in Fortran notation like `1d0`
    are left for the caller)."""
    out = {}
    with open(path) as fh:
        for line in fh:
            t = line.split("!")[0].split()
            if len(t) >= 2:
                out[t[0]] = t[1]
    return out


def fortran_float(s):
    return float(str(s).lower().replace("d", "e"))


# the keys of one dataset stored in a bundle (`save_bundle` / `load_bundle`)
_ARRAYS = ("l", "f", "rc_state", "e", "r", "dr", "phi", "tphi", "ptilde", "kij") + tuple(_FUNCS.values())
_SCALARS = ("Z", "core", "valence", "rpaw", "rcomp")


def save_bundle(path, datasets, symbols, coords, params):
    """Writes datasets (symbol -> dict of `read_dataset`), a geometry and the
    run parameters into one compressed .npz."""
    out = {"symbols": np.array(symbols), "coords": coords,
           "param_keys": np.array(list(params.keys())), "param_vals": np.array(list(params.values())),
           "species": np.array(sorted(datasets))}
    for s, d in datasets.items():
        for k in _ARRAYS:
            out[f"{s}/{k}"] = d[k]
        for k in _SCALARS:
            out[f"{s}/{k}"] = np.float64(d[k])
        out[f"{s}/shape_type"] = np.array(d["shape_type"])
        out[f"{s}/ids"] = np.array(d["ids"])
    np.savez_compressed(path, **out)


def load_bundle(path):
    """Inverse of `save_bundle`: (datasets, symbols, coords, params)."""
    z = np.load(path)
    datasets = {}
    for s in z["species"]:
        s = str(s)
        d = {"symbol": s}
        for k in _ARRAYS:
            d[k] = z[f"{s}/{k}"]
        for k in _SCALARS:
            d[k] = float(z[f"{s}/{k}"])
        d["shape_type"] = str(z[f"{s}/shape_type"])
        d["ids"] = [str(v) for v in z[f"{s}/ids"]]
        datasets[s] = d
    params = {str(k): str(v) for k, v in zip(z["param_keys"], z["param_vals"])}
    return datasets, [str(v) for v in z["symbols"]], z["coords"], params


def _fmt(a, per_line=3):
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    lines = []
    for i in range(0, a.size, per_line):
        lines.append(" ".join(f"{v: .17e}" for v in a[i:i + per_line]))
    return "\n".join(lines)


def write_dataset(path, d):
    """Writes a dataset dict (the keys `read_dataset` returns) as PAW-XML with
    one shared radial grid; `read_dataset` reads it back bit for bit."""
    out = ['<?xml version="1.0"?>', '<paw_dataset version="0.7">',
           f'<atom symbol="{d["symbol"]}" Z="{d["Z"]!r}" core="{d["core"]!r}" valence="{d["valence"]!r}"/>',
           f'<paw_radius rc="{d["rpaw"]!r}"/>', "<valence_states>"]
    for sid, l, f, rc, e in zip(d["ids"], d["l"], d["f"], d["rc_state"], d["e"]):
        out.append(f'  <state l="{int(l)}" f="{float(f)!r}" rc="{float(rc)!r}" e="{float(e)!r}" id="{sid}"/>')
    out.append("</valence_states>")
    n = len(d["r"])
    out.append(f'<radial_grid eq="{d.get("grid_eq", "")}" istart="0" iend="{n - 1}" id="g1">')
    out += ["  <values>", _fmt(d["r"]), "  </values>", "  <derivatives>", _fmt(d["dr"]), "  </derivatives>",
            "</radial_grid>"]
    out.append(f'<shape_function type="{d["shape_type"]}" rc="{d["rcomp"]!r}"/>')
    for tag, key in _FUNCS.items():
        out += [f'<{tag} grid="g1">', _fmt(d[key]), f"</{tag}>"]
    for i, sid in enumerate(d["ids"]):
        for tag, key in (("ae_partial_wave", "phi"), ("pseudo_partial_wave", "tphi"), ("projector_function", "ptilde")):
            out += [f'<{tag} state="{sid}" grid="g1">', _fmt(d[key][i]), f"</{tag}>"]
    out += ["<kinetic_energy_differences>", _fmt(d["kij"]), "</kinetic_energy_differences>", "</paw_dataset>"]
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


def read_folder(folder):
    """The reference's input folder: `pawfiles` (element symbol and dataset
    file per line), the datasets, `cnt.ini` and `dim_paw.inp`.  Returns
    (datasets, symbols, coords, params) like `load_bundle`."""
    import os

    datasets = {}
    with open(os.path.join(folder, "pawfiles")) as fh:
        for line in fh:
            t = line.split()
            if len(t) >= 2:
                datasets[t[0]] = read_dataset(os.path.join(folder, t[1]))
    symbols, coords = read_geometry(os.path.join(folder, "cnt.ini"))
    missing = sorted(set(symbols) - set(datasets))
    if missing:
        raise ValueError(f"{folder}: no dataset in pawfiles for {missing}")
    return datasets, symbols, coords, read_parameters(os.path.join(folder, "dim_paw.inp"))


def write_folder(folder, datasets, symbols, coords, params):
    """Lays out an input folder as the reference reads it: one `<symbol>.xml`
    per dataset listed in `pawfiles`, `cnt.ini` and `dim_paw.inp`."""
    import os

    with open(os.path.join(folder, "pawfiles"), "w") as fh:
        for s, d in datasets.items():
            write_dataset(os.path.join(folder, f"{s}.xml"), d)
            fh.write(f"{s}     {s}.xml\n")
    with open(os.path.join(folder, "cnt.ini"), "w") as fh:
        for s, p in zip(symbols, coords):
            fh.write(f" {s} {float(p[0])!r} {float(p[1])!r} {float(p[2])!r}\n")
    with open(os.path.join(folder, "dim_paw.inp"), "w") as fh:
        for k, v in params.items():
            fh.write(f"{k} {v}\n")
