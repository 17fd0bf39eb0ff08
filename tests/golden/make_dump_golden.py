"""Generate tests/golden/dump_*.npz: dump files written by the reference's
own dump() (src/dump.c, called from do_step; oracle/ref_md.c) during short
constant-energy runs from the starts of the md_* fixtures.

Each fixture holds the name of the md_* fixture it starts from, the run
length, the dump level, interval, records per file and title, and every
file the reference wrote (raw bytes, key "file:<name>").  The reference is
built without XDR (rpc/xdr.h is absent here), so these are native LP64
files.

usage: python tests/golden/make_dump_golden.py [--only NAME]
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from moldy_gb300 import system as S  # noqa: E402
from moldy_gb300.dynamics import Dynamics, MDState  # noqa: E402
from oracle import md  # noqa: E402

CASES = [
    # name, md fixture, steps, level, interval, ndumps, title
    ("dump_water864", "md_water864", 30, 11, 5, 4, "rigid water, 216 molecules"),
    ("dump_argon500", "md_argon500", 50, 3, 10, 10, "argon fcc 500"),
    ("dump_rocksalt512", "md_rocksalt512", 30, 9, 10, 2, "rock salt 512"),
    ("dump_waterwall", "md_waterwall", 30, 11, 10, 4, "water over a framework"),
]


def load_md(name):
    sysm, z = S.load_npz(os.path.join(HERE, name + ".npz"))
    dyn = Dynamics(z["md_mass"], z["md_inertia"].reshape(-1, 3), z["md_rdof"], float(z["md_step"]),
                   bool(z["md_nosym"]))
    return sysm, dyn, MDState(z["c_of_m0"], z["mom0"], z["quat0"], z["amom0"])


def main():
    subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    for name, src, steps, level, interval, ndumps, title in CASES:
        if only is not None and name != only:
            continue
        sysm, dyn, st0 = load_md(src)
        _, _, _, files = md.run(sysm, dyn, st0, steps, dump=("run%02d.dmp", level, interval, ndumps, title))
        arrs = {"file:" + k: np.frombuffer(v, np.uint8) for k, v in files.items()}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), md_fixture=src, steps=steps, level=level,
                            interval=interval, ndumps=ndumps, title=title, **arrs)
        print(name, {k: len(v) for k, v in files.items()})


if __name__ == "__main__":
    main()
