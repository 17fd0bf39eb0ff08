"""The C ABI without a GPU: the library loads, exports every function the
headers under include/ declare, and the reference-compatible struct layouts
of include/moldy_ref_abi.h match the reference's own src/structs.h."""
import os
import re
import subprocess
import tempfile

import pytest

from conftest import ROOT
from oracle.ref import source_dir

INCLUDE = os.path.join(ROOT, "include")
REF_SRC = source_dir()


def declared_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(\w+)\s*\([^;{]*\)\s*;", text, flags=re.M):
            name = m.group(1)
            if name not in ("if", "while", "for", "return", "sizeof"):
                names.add(name)
    return sorted(names)


@pytest.fixture(scope="module")
def libpath():
    from moldy_gb300 import build
    return build.build()


def test_headers_declare_the_reference_entry_points():
    names = declared_functions()
    for n in ("force_calc", "ewald", "poteval", "mdgpu_forces", "mdgpu_force_calc", "mdgpu_ewald"):
        assert n in names


def test_library_exports_every_declared_function(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_library_loads_and_binds_without_a_gpu(libpath):
    from moldy_gb300 import _lib
    L = _lib.load()
    for n in _lib.EXPORTS:
        assert hasattr(L, n), n
    # context creation reports the missing device instead of crashing
    import ctypes as C
    ctx = C.c_void_p()
    st = L.mdgpu_create(C.byref(ctx), 0, _lib.MIXED)
    import torch
    if not torch.cuda.is_available():
        assert st == 2   # MDGPU_E_CUDA


def test_poteval_matches_the_oracle_on_the_host(libpath):
    """poteval is host arithmetic (used for set-up constants): it must equal
    the oracle's restatement of src/force.c:632-650 bit for bit."""
    import numpy as np
    from moldy_gb300 import _lib
    from moldy_gb300.forcefield import poteval
    from oracle import port
    port.build()
    rng = np.random.default_rng(3)
    for ptype in (0, 1, 2, 3, 4, 6):
        for alpha in (-1.0, 0.0, 0.35):
            p = rng.uniform(0.5, 3.0, 8)
            r = float(rng.uniform(0.8, 9.0))
            q = float(rng.uniform(-5e4, 5e4))
            assert poteval(p, r, ptype, q, alpha) == port.poteval(p, r, ptype, q, alpha)


LAYOUT_C = r"""
#include <stdio.h>
#include <stddef.h>
#include HDR
#define P(T, f) printf("%s.%s %zu\n", #T, #f, offsetof(T, f));
int main(void) {
  P(contr_mt, istep) P(contr_mt, molpbc) P(contr_mt, surface_dipole) P(contr_mt, spare)
  P(contr_mt, ewald_accuracy) P(contr_mt, strict_cutoff) P(contr_mt, seed) P(contr_mt, page_width)
  P(contr_mt, dump_level) P(contr_mt, begin_rdf) P(contr_mt, rdf_interval) P(contr_mt, cutoff)
  P(contr_mt, subcell) P(contr_mt, alpha) P(contr_mt, k_cutoff) P(contr_mt, limit) P(contr_mt, cpu_limit)
  P(system_mt, nsites) P(system_mt, max_id) P(system_mt, ptype) P(system_mt, n_potpar)
  P(system_mt, c_of_m) P(system_mt, h) P(system_mt, rsmom)
  P(spec_mt, nsites) P(spec_mt, nmols) P(spec_mt, framework) P(spec_mt, name) P(spec_mt, site_id)
  P(spec_mt, p_f_sites) P(spec_mt, quat)
  P(pot_mt, p)
  printf("sizeof %zu %zu %zu %zu\n", sizeof(contr_mt), sizeof(system_mt), sizeof(spec_mt), sizeof(pot_mt));
  return 0;
}
"""


@pytest.mark.skipif(REF_SRC is None, reason="reference sources not present")
def test_struct_layout_matches_the_reference_header():
    outs = []
    with tempfile.TemporaryDirectory() as td:
        # defs.h includes a version.h that the reference's git hook writes
        open(os.path.join(td, "version.h"), "w").write(
            '#define REVISION "t"\n#define REVISION_DATE "t"\n#define REVISION_STATE "t"\n')
        for tag, hdr, inc in (("ours", '"moldy_ref_abi.h"', INCLUDE), ("ref", '"structs.h"', REF_SRC)):
            src = os.path.join(td, tag + ".c")
            open(src, "w").write(LAYOUT_C.replace("HDR", hdr))
            exe = os.path.join(td, tag)
            subprocess.run(["gcc", "-w", "-I", td, "-I", inc, "-DHAVE_VOID_PTRS", "-DSTDC_HEADERS", src,
                            "-o", exe], check=True)
            outs.append(subprocess.run([exe], capture_output=True, text=True, check=True).stdout)
    assert outs[0] == outs[1]
