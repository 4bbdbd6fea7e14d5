"""Generates tests/golden/jth_naphthalene.npz: the reference's naphthalene
example (its `naph/` input folder) as one bundle — the JTH LDA PAW datasets
of C and H (`C.LDA_PW-JTH.xml`, `H.LDA_PW-JTH.xml`, read by
`opaw_tddft_gb300.pawxml.read_dataset`), the geometry `cnt.ini` and the run
parameters `dim_paw.inp`.  The radial arrays are kept up to r = 20 Bohr: the
projectors and partial-wave differences vanish beyond 1.6 Bohr, the densities
are below 1e-13 there and the local potential equals -Z_val / r to 1e-7
relative from 3 Bohr on (the set-up chain continues it analytically).

Usage: python tests/golden/make_jth_fixture.py [reference naph folder]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
R_KEEP = 20.0


def main(src):
    sys.path.insert(0, ROOT)
    import __graft_entry__

    __graft_entry__.load_package()
    from opaw_tddft_gb300 import pawxml

    files = {}
    for line in open(os.path.join(src, "pawfiles")):
        t = line.split()
        if len(t) >= 2:
            files[t[0]] = t[1]
    datasets = {}
    for sym, fn in files.items():
        d = pawxml.read_dataset(os.path.join(src, fn))
        n = int(np.searchsorted(d["r"], R_KEEP)) + 1
        for k in ("r", "dr", "ae_core", "ps_core", "ps_valence", "zero_potential", "vloc_blochl"):
            d[k] = d[k][:n]
        for k in ("phi", "tphi", "ptilde"):
            d[k] = d[k][:, :n]
        datasets[sym] = d
    symbols, coords = pawxml.read_geometry(os.path.join(src, "cnt.ini"))
    params = pawxml.read_parameters(os.path.join(src, "dim_paw.inp"))
    out = os.path.join(HERE, "jth_naphthalene.npz")
    pawxml.save_bundle(out, datasets, symbols, coords, params)
    print(out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/naph")
