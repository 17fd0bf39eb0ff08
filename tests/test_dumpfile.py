"""Dump-file format against files the reference's own dump() wrote
(tests/golden/make_dump_golden.py): the reader parses them, and the
library's writer, given the same records and header data, writes the same
bytes -- apart from the bytes the reference leaves uninitialised after the
title and species-name terminators, and the two wall-clock stamps."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

CASES = ["dump_water864", "dump_argon500", "dump_rocksalt512", "dump_waterwall"]


def _fixture(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    files = {k[5:]: z[k].tobytes() for k in z.files if k.startswith("file:")}
    return z, files


def _md(name):
    from moldy_gb300 import system
    from moldy_gb300.dynamics import Dynamics
    sysm, z = system.load_npz(os.path.join(GOLDEN, name + ".npz"))
    dyn = Dynamics(z["md_mass"], z["md_inertia"].reshape(-1, 3), z["md_rdof"], float(z["md_step"]),
                   bool(z["md_nosym"]))
    return sysm, dyn


def _mask(data, nspecies):
    """Byte positions compared: all but the tails after the title and name
    terminators and the timestamp/dump_init fields (offsets 176-191)."""
    keep = np.ones(len(data), bool)
    t = data.index(b"\0")
    keep[t:128] = False
    keep[176:192] = False
    for k in range(nspecies):
        o = 208 + 16 + 68 * k + 36
        n = data.index(b"\0", o)
        keep[n:o + 32] = False
    return keep


def _read(tmp_path, fname, data):
    from moldy_gb300.dumpfile import read_dump
    p = tmp_path / fname
    p.write_bytes(data)
    return read_dump(str(p))


@pytest.mark.parametrize("name", CASES)
def test_reader_on_reference_files(name, tmp_path):
    from moldy_gb300.dumpfile import dump_size, split_record
    z, files = _fixture(name)
    sysm, dyn = _md(str(z["md_fixture"]))
    level, interval, nd = int(z["level"]), int(z["interval"]), int(z["ndumps"])
    nq = int(sum(sp.nmols for k, sp in enumerate(sysm.species) if dyn.rdof[k] > 0))
    total = 0
    for i, fname in enumerate(sorted(files)):
        f = _read(tmp_path, fname, files[fname])
        assert not f.xdr and f.vsn == "2.27" and f.title == str(z["title"])
        assert (f.dump_level, f.dump_interval, f.maxdumps) == (level, interval, nd)
        assert f.istep == 1 + i * nd * interval
        assert f.dump_size == dump_size(level, sysm.nmols, nq)
        assert f.sysinfo_size == 16 + 68 * len(sysm.species)
        assert (f.nmols, f.nmols_r) == (sysm.nmols, nq)
        assert abs(f.deltat - dyn.step * interval) < 1e-6 * dyn.step * interval
        assert [s["nmols"] for s in f.species] == [sp.nmols for sp in sysm.species]
        total += f.ndumps
        parts = split_record(f.records[0], level, sysm.nmols, nq)
        if level & 1:
            np.testing.assert_allclose(parts["h"], sysm.h.astype(np.float32))
            assert parts["ts"][0] == 1.0
        if level & 2:
            assert not parts["hmom"].any() and parts["tsmom"][0] == 0.0
    assert total == (int(z["steps"]) - 1) // interval + 1


@pytest.mark.parametrize("name", CASES)
def test_writer_matches_reference_bytes(name, tmp_path):
    from moldy_gb300.dumpfile import DumpWriter, species_info
    z, files = _fixture(name)
    sysm, dyn = _md(str(z["md_fixture"]))
    level, interval, nd = int(z["level"]), int(z["interval"]), int(z["ndumps"])
    nq = int(sum(sp.nmols for k, sp in enumerate(sysm.species) if dyn.rdof[k] > 0))
    refs = [_read(tmp_path, fn, files[fn]) for fn in sorted(files)]
    sp = species_info(sysm, dyn, names=[f"spec{k}" for k in range(len(sysm.species))])
    out = tmp_path / "ours"
    out.mkdir()
    with DumpWriter(str(out / "run%02d.dmp"), sp, level, interval, nd, dyn.step, sysm.nmols, nq,
                    istep=1, title=str(z["title"])) as w:
        for r in refs:
            for rec in r.records:
                w.append(rec)
    for fname in sorted(files):
        a = files[fname]
        b = (out / fname).read_bytes()
        assert len(a) == len(b)
        keep = _mask(a, len(sysm.species))
        A, B = np.frombuffer(a, np.uint8), np.frombuffer(b, np.uint8)
        bad = np.nonzero((A != B) & keep)[0]
        assert bad.size == 0, f"{fname}: bytes differ at {bad[:10]}"


def test_xdr_round_trip(tmp_path):
    from moldy_gb300.dumpfile import DumpWriter, read_dump, species_info
    z, files = _fixture("dump_water864")
    sysm, dyn = _md(str(z["md_fixture"]))
    ref = _read(tmp_path, "ref.dmp", files["run00.dmp"])
    sp = species_info(sysm, dyn)
    with DumpWriter(str(tmp_path / "x%d.xdr"), sp, ref.dump_level, ref.dump_interval, 8, dyn.step,
                    ref.nmols, ref.nmols_r, istep=1, title="xdr", xdr=True, dump_init=12345,
                    restart_timestamp=777) as w:
        for rec in ref.records:
            w.append(rec)
    x = read_dump(str(tmp_path / "x0.xdr"))
    assert x.xdr and x.vsn == "2.27(XDR)" and x.title == "xdr"
    assert (x.ndumps, x.dump_size, x.dump_init, x.restart_timestamp) == (4, ref.dump_size, 12345, 777)
    assert x.sysinfo_size == 16 + 68
    np.testing.assert_array_equal(x.records, ref.records)
    # XDR_DUMP_SIZE + XDR_SYSINFO_SIZE + records (src/xdr.h:117-123)
    assert os.path.getsize(tmp_path / "x0.xdr") == 184 + 84 + 4 * ref.dump_size * 4
    assert x.species[0]["name"] == sp[0]["name"]


def test_template_rules(tmp_path):
    from moldy_gb300._lib import MdgpuError
    from moldy_gb300.dumpfile import DumpWriter
    sp = [dict(inertia=[0, 0, 0], mass=1.0, dipole=0.0, charge=0.0, nmols=2, rdof=0, framework=0, name="a")]
    with pytest.raises(MdgpuError, match="integer conversion"):
        DumpWriter(str(tmp_path / "bad%s"), sp, 1, 1, 2, 0.01, 2, 0)
    # no conversion: the file number is appended
    with DumpWriter(str(tmp_path / "plain"), sp, 1, 1, 2, 0.01, 2, 0) as w:
        assert w.append(np.zeros(w.size, np.float32)).endswith("plain0")
        w.append(np.zeros(w.size, np.float32))
        assert w.append(np.zeros(w.size, np.float32)).endswith("plain1")
    # an existing file is not overwritten
    with DumpWriter(str(tmp_path / "plain"), sp, 1, 1, 2, 0.01, 2, 0) as w:
        with pytest.raises(MdgpuError, match="exists"):
            w.append(np.zeros(w.size, np.float32))


def _xdr_expected(title, istep, interval, level, maxdumps, records, timestamp, dump_init, rts, deltat,
                  nmols, nmols_r, species):
    """A dump file as the XDR standard (RFC 4506: big-endian 4-byte units,
    fixed-length opaque data padded to a multiple of 4) encodes the
    reference's XDR routines' field order, written here from those rules
    alone: xdr_dump (src/xdr.c:150-157) -- opaque title and version (128 +
    16 bytes), xdr_long istep and dump_interval, xdr_int dump_level,
    maxdumps, ndumps, dump_size, xdr_u_long timestamp, dump_init,
    restart_timestamp, sysinfo_size; xdr_dump_sysinfo_2_23
    (src/xdr.c:168-182) -- xdr_float deltat, xdr_int nmols, nmols_r,
    nspecies, per species xdr_float inertia[3], mass, dipole, charge, xdr_int
    nmols, rdof, framework, opaque name (32 bytes); then each record as
    dump_size xdr_floats (src/dump.c:263-264)."""
    import struct

    def opaque(b, n):
        b = b[:n] + b"\0" * (n - len(b[:n]))
        return b + b"\0" * (-n % 4)
    nd, size = records.shape
    out = opaque(title.encode(), 128) + opaque(b"2.27(XDR)", 16)
    out += struct.pack(">ll", istep, interval)
    out += struct.pack(">iiii", level, maxdumps, nd, size)
    out += struct.pack(">LLLL", timestamp, dump_init, rts, 16 + 68 * len(species))
    out += struct.pack(">fiii", deltat, nmols, nmols_r, len(species))
    for s in species:
        out += struct.pack(">ffffff", *s["inertia"], s["mass"], s["dipole"], s["charge"])
        out += struct.pack(">iii", s["nmols"], s["rdof"], s["framework"])
        out += opaque(s["name"].encode(), 32)
    for r in records:
        out += struct.pack(">%df" % size, *[float(v) for v in r])
    return out


def test_xdr_bytes_follow_rfc4506(tmp_path):
    """The XDR dump file, byte for byte, against an encoder written from the
    XDR standard and the reference's field order (the reference's own XDR
    build needs a system rpc/xdr.h, absent here, so its files cannot be
    made): only the wall-clock stamp is taken from the file."""
    import struct

    from moldy_gb300.dumpfile import DumpWriter, species_info
    z, files = _fixture("dump_water864")
    sysm, dyn = _md(str(z["md_fixture"]))
    ref = _read(tmp_path, "ref.dmp", files["run00.dmp"])
    sp = species_info(sysm, dyn)
    with DumpWriter(str(tmp_path / "x%d.xdr"), sp, ref.dump_level, ref.dump_interval, 8, dyn.step,
                    ref.nmols, ref.nmols_r, istep=3, title="rfc4506 check", xdr=True, dump_init=424242,
                    restart_timestamp=99) as w:
        for rec in ref.records:
            w.append(rec)
    got = (tmp_path / "x0.xdr").read_bytes()
    stamp = struct.unpack_from(">L", got, 168)[0]
    spf = [dict(s, inertia=[float(np.float32(v)) for v in s["inertia"]]) for s in sp]
    for s in spf:
        for k in ("mass", "dipole", "charge"):
            s[k] = float(np.float32(s[k]))
    want = _xdr_expected("rfc4506 check", 3, ref.dump_interval, ref.dump_level, 8, ref.records, stamp,
                         424242, 99, float(np.float32(dyn.step * ref.dump_interval)), ref.nmols, ref.nmols_r, spf)
    assert len(got) == len(want)
    bad = [i for i in range(len(got)) if got[i] != want[i]]
    assert not bad, f"bytes differ at {bad[:10]}"


def test_restart_state_reads_the_reference_restart_file():
    """moldy_gb300.dynamics.restart_state takes the dynamic state out of a
    restart file the reference's write_restart produced (native format):
    bit for bit the state the reference's run reached."""
    from moldy_gb300 import system
    from moldy_gb300.dynamics import restart_state
    sysm, z = system.load_npz(os.path.join(GOLDEN, "md_restart_water864.npz"))
    st = restart_state(z["restart_file"].tobytes(), len(sysm.species), sysm.nmols, len(z["quat0"]))
    for got, key in ((st.c_of_m, "c_of_m_restart"), (st.mom, "mom_restart"), (st.quat, "quat_restart"),
                     (st.amom, "amom_restart")):
        np.testing.assert_array_equal(got, z[key])
