"""Run the reference's own force_calc/ewald through oracle/_ref/moldy_ref_harness.

TEST INFRASTRUCTURE ONLY: used to validate the C restatement and to generate
golden fixtures where the reference sources are present.  One configuration per
process, because force_calc and ewald keep first-call statics
(src/force.c:1146-1149, src/ewald.c:352-355).
"""
from __future__ import annotations

import os
import re
import subprocess
import tempfile
from dataclasses import dataclass
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")


def available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "moldy_ref_harness"))


def source_dir() -> Optional[str]:
    """The reference's src/ directory: MOLDY_SRC when set, else the one
    oracle/build_ref.sh last built from (recorded in oracle/_ref/SRC_DIR);
    None when neither exists (as on a machine without the sources)."""
    cand = os.environ.get("MOLDY_SRC")
    if not cand:
        try:
            with open(os.path.join(REF_DIR, "SRC_DIR")) as f:
                cand = f.read().strip()
        except OSError:
            return None
    return cand if os.path.isfile(os.path.join(cand, "force.c")) else None


def build() -> bool:
    """Build oracle/_ref from the reference sources if they are present."""
    subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")], check=True,
                   stdout=subprocess.DEVNULL)
    return available()


@dataclass
class RefResult:
    force_real: np.ndarray      # [3, N]
    pe_real: float
    stress_real: np.ndarray     # [3, 3] upper triangle filled
    force_ewald: np.ndarray     # [3, N]
    pe_ewald: float
    stress_ewald: np.ndarray
    pairs: Optional[np.ndarray]  # [P, 3] int32 (isite, jsite, image index 0..26)
    stdout: str
    t_force: Optional[float] = None
    t_ewald: Optional[float] = None
    rdf: Optional[np.ndarray] = None   # the reference's float RDF histogram (rdf_ptr layout)

    def notes(self):
        return [l.strip() for l in self.stdout.splitlines() if l.strip().startswith("*")]


def run(sysm, want_pairs: bool = False, repeats: int = 1, fast: bool = False,
        rdf: Optional[tuple] = None) -> RefResult:
    """rdf = (limit, nbins): also accumulate the reference's RDF histogram on
    the first force_calc call."""
    from moldy_gb300.system import write_mdsys
    exe = os.path.join(REF_DIR, "moldy_ref_harness_fast" if fast else "moldy_ref_harness")
    n = sysm.nsites
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.mdsys"), os.path.join(td, "out.bin")
        write_mdsys(fin, sysm, want_pairs)
        env = dict(os.environ)
        if rdf is not None:
            env["MDGPU_REF_RDF"] = f"{float(rdf[0])!r} {int(rdf[1])}"
        cp = subprocess.run([exe, fin, fout, str(repeats)], capture_output=True, text=True, env=env)
        if cp.returncode != 0:
            raise RuntimeError(f"reference harness failed ({cp.returncode}): {cp.stdout[-2000:]}{cp.stderr[-2000:]}")
        raw = open(fout, "rb").read()
    d = np.frombuffer(raw, dtype="<f8", count=2 * (3 * n + 10))
    fr = d[:3 * n].reshape(3, n).copy()
    per = d[3 * n]
    sr = d[3 * n + 1:3 * n + 10].reshape(3, 3).copy()
    o = 3 * n + 10
    fe = d[o:o + 3 * n].reshape(3, n).copy()
    pee = d[o + 3 * n]
    se = d[o + 3 * n + 1:o + 3 * n + 10].reshape(3, 3).copy()
    off = 8 * 2 * (3 * n + 10)
    npairs = int(np.frombuffer(raw, dtype="<i8", count=1, offset=off)[0])
    pairs = None
    if npairs >= 0:
        pairs = np.frombuffer(raw, dtype="<i4", count=3 * npairs, offset=off + 8).reshape(-1, 3).copy()
    off += 8 + (12 * npairs if npairs > 0 else 0)
    hist = None
    if rdf is not None:
        size = int(np.frombuffer(raw, dtype="<i8", count=1, offset=off)[0])
        hist = np.frombuffer(raw, dtype="<f4", count=size, offset=off + 8).copy()
    tf = te = None
    m = re.search(r"HARNESS_TIMING force_calc (\S+) ewald (\S+)", cp.stdout)
    if m:
        tf, te = float(m.group(1)), float(m.group(2))
    return RefResult(fr, float(per), sr, fe, float(pee), se, pairs, cp.stdout, tf, te, hist)
