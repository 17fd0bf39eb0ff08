"""Generate the radial-distribution fixtures tests/golden/rdf_*.npz from the
reference itself: the float histogram its force_calc accumulates on an RDF
step (rdf_inner/rdf_accum, src/force.c:1010-1103, src/rdf.c:94-107; driven by
oracle/ref_harness.c with MDGPU_REF_RDF), for one configuration each.

usage: python tests/golden/make_rdf_golden.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from moldy_gb300 import system as S  # noqa: E402
from oracle import ref  # noqa: E402

CASES = [
    ("rdf_water864", lambda: S.water(nside=6, seed=3), 9.0, 90),
    ("rdf_water864_strict", lambda: S.water(nside=6, seed=3, strict=True), 8.0, 100),
    ("rdf_water864_molpbc", lambda: S.water(nside=6, seed=3, molpbc=True), 9.0, 90),
    ("rdf_argon500", lambda: S.argon_fcc(), 12.0, 120),
    ("rdf_rocksalt512", lambda: S.rock_salt(ncell=4), 10.0, 100),
]


def main():
    ref.build()
    for name, make, limit, nbins in CASES:
        sysm = make()
        r = ref.run(sysm, rdf=(limit, nbins))
        S.save_npz(os.path.join(HERE, name + ".npz"), sysm, rdf_limit=limit, rdf_nbins=nbins, ref_rdf=r.rdf)
        print(name, sysm.nsites, "sites", r.rdf.size, "bins", float(r.rdf.sum()))


if __name__ == "__main__":
    main()
