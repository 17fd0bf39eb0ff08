"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run where the reference sources are available (it builds them in place with
oracle/build_ref.sh); the GPU machine only reads the committed .npz files.

Each fixture holds one input configuration (a System, see
moldy_gb300/system.py) and the reference's own outputs on it: real-space and
reciprocal-space site forces, energies and stress (oracle/ref_harness.c), the
logged constants (subcells, neighbour cells, k-vectors, self-energy,
intramolecular correction) and a digest of the evaluated pair set (the full
canonical key list for the smaller cases).

Two families:
  ex_*   the reference's own example runs (src/examples/control.*), set up by
         the reference's start_up and make_sites (oracle/ref_examples.c);
  syn_*  seeded synthetic workloads with the shapes of the measured configs.

usage: python tests/golden/make_golden.py
"""
import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from moldy_gb300 import system as S  # noqa: E402
from moldy_gb300 import pairset  # noqa: E402
from oracle import ref  # noqa: E402

FULL_KEYS_MAX = 60000


def notes_dict(notes):
    d = {}
    for line in notes:
        m = re.search(r"MD cell divided into (\d+) subcells \((\d+)x(\d+)x(\d+)\)", line)
        if m:
            d["ncells"], d["nx"], d["ny"], d["nz"] = map(int, m.groups())
        m = re.search(r"Neighbour list contains (\d+) cells", line)
        if m:
            d["nabor_cells"] = int(m.group(1))
        m = re.search(r"Ewald self-energy = (\S+) kJ/mol", line)
        if m:
            d["self_energy_kjmol"] = float(m.group(1))
        m = re.search(r"(\d+) K-vectors included", line)
        if m:
            d["nkvec"] = int(m.group(1))
        m = re.search(r"Intramolecular potential energy correction = (\S+)", line)
        if m:
            d["eintra_kjmol"] = float(m.group(1))
    return d


def make(name, sysm):
    r = ref.run(sysm, want_pairs=True)
    keys = pairset.keys_from_triplets(r.pairs)
    cnt, dig = pairset.digest(keys)
    nd = notes_dict(r.notes())
    extra = dict(force_real=r.force_real, pe_real=r.pe_real, stress_real=r.stress_real,
                 force_ewald=r.force_ewald, pe_ewald=r.pe_ewald, stress_ewald=r.stress_ewald,
                 npairs=cnt, pair_digest=np.array([dig], np.uint64),
                 notes=np.array(r.notes()))
    for k, v in nd.items():
        extra["log_" + k] = v
    if cnt <= FULL_KEYS_MAX:
        extra["pair_keys"] = keys
    path = os.path.join(HERE, name + ".npz")
    S.save_npz(path, sysm, **extra)
    print(f"{name}: N={sysm.nsites} pairs={cnt} notes={nd} -> {os.path.getsize(path)} B")


def examples():
    exe = os.path.join(ROOT, "oracle", "_ref", "moldy_ref_examples")
    for c in ["water", "tips2", "tip4p", "mgclh2o", "argon", "quartz", "clay"]:
        with tempfile.TemporaryDirectory() as td:
            wd = os.path.join(td, "ex")
            shutil.copytree(os.path.join(ref.source_dir(), "examples"), wd)
            out = os.path.join(wd, c + ".mdsys")
            subprocess.run([exe, "control." + c, out], cwd=wd, check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            make("ex_" + c, S.read_mdsys(out, "ex_" + c))


def synthetic():
    make("syn_argon500_strict", S.argon_fcc())
    make("syn_water2048", S.water(nside=8))
    make("syn_water864_strict", S.water(nside=6, strict=True))
    make("syn_water864_molpbc", S.water(nside=6, molpbc=True))
    make("syn_water864_mcy", S.water(nside=6, model="mcy"))
    make("syn_rocksalt512", S.rock_salt(ncell=4))
    make("syn_generic216", S.generic_ions(S.GENPOT))
    make("syn_hiw216", S.generic_ions(S.HIWPOT))
    make("syn_morse216", S.generic_ions(S.MORPOT))


if __name__ == "__main__":
    if not ref.build():
        sys.exit("reference sources not found; set MOLDY_SRC")
    examples()
    synthetic()
