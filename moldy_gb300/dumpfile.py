"""Dump files of the reference (src/dump.c): trajectory records written from
the GPU dynamics run.

A dump record is the FP32 conversion of the state after a step
(dump_convert, src/dump.c:550-620), its parts selected by the bits of the
dump level: 1 positions/quaternions/h/ts/pe, 2 velocities, 8 forces,
torques and stress.  :meth:`MolecularDynamics.run_dump` converts records on
the GPU; :class:`DumpWriter` writes them into the reference's sequence of
files (through the library's C writer, native or XDR layout) and
:func:`read_dump` reads such a file back, whichever program wrote it.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import struct
from typing import Dict, List, Optional

import numpy as np

from . import _lib

L_NAME, L_VSN, L_SPEC = 128, 16, 32
_HDR_NATIVE = struct.Struct("<128s16sqqiiiiQQQQ")     # dump_mt, LP64
_HDR_XDR = struct.Struct(">128s16siiiiiiIIII")         # xdr_dump, src/xdr.c:150-157
_SYS_NATIVE, _SYS_XDR = struct.Struct("<fiii"), struct.Struct(">fiii")
_MOL_NATIVE, _MOL_XDR = struct.Struct("<6f3i32s"), struct.Struct(">6f3i32s")


def dump_size(level: int, nmols: int, nmols_r: int) -> int:
    """Floats per record (DUMP_SIZE, src/defs.h:294-297)."""
    return ((level & 1) * (3 * nmols + 4 * nmols_r + 11) + (level >> 1 & 1) * (3 * nmols + 3 * nmols_r + 10) +
            (level >> 3 & 1) * (3 * nmols + 3 * nmols_r + 9))


def split_record(rec: np.ndarray, level: int, nmols: int, nmols_r: int) -> Dict[str, np.ndarray]:
    """Named parts of one record, in dump_convert's order."""
    out, o = {}, 0

    def take(name, n, shape=None):
        nonlocal o
        a = np.asarray(rec[o:o + n])
        out[name] = a.reshape(shape) if shape else a
        o += n

    if level & 1:
        take("c_of_m", 3 * nmols, (nmols, 3))
        take("quat", 4 * nmols_r, (nmols_r, 4))
        take("h", 9, (3, 3))
        take("ts", 1)
        take("pe", 1)
    if level & 2:
        take("vel", 3 * nmols, (nmols, 3))
        take("avel", 3 * nmols_r, (nmols_r, 3))
        take("hmom", 9, (3, 3))
        take("tsmom", 1)
    if level & 8:
        take("force", 3 * nmols, (nmols, 3))
        take("torque", 3 * nmols_r, (nmols_r, 3))
        take("stress", 9, (3, 3))
    return out


def species_info(sysm, dyn, names: Optional[List[str]] = None) -> List[dict]:
    """The per-species record of the dump header (mol_mt): principal
    moments, mass, dipole |sum q p| over the principal-frame sites of a
    rotating species (0 for one without rotation, src/startup.c:571-580),
    molecular charge, counts and name."""
    out = []
    for k, sp in enumerate(sysm.species):
        q = np.asarray(sysm.site_charge, np.float64)[sp.site_id]
        rot = int(dyn.rdof[k]) > 0
        dip = float(np.sqrt(np.sum(((np.asarray(sp.p_f_sites, np.float64) * q[:, None]).sum(0)) ** 2))) if rot else 0.0
        out.append(dict(inertia=[float(x) for x in np.asarray(dyn.inertia).reshape(-1, 3)[k]],
                        mass=float(dyn.mass[k]), dipole=dip, charge=float(q.sum()), nmols=int(sp.nmols),
                        rdof=int(dyn.rdof[k]), framework=int(bool(sp.framework)),
                        name=(names[k] if names else sp.name)))
    return out


class DumpWriter:
    """A sequence of dump files (mdgpu_dump_open/append/close).

    ``template`` holds the file number as one integer conversion ("%d" is
    appended when it has none); ``istep`` is the step of the first record.
    """

    def __init__(self, template: str, species: List[dict], level: int, interval: int, maxdumps: int,
                 step: float, nmols: int, nmols_r: int, istep: int = 1, title: str = "", xdr: bool = False,
                 dump_init: int = 0, restart_timestamp: int = 0):
        self.L = _lib.load()
        arr = (_lib.DumpSpecies * len(species))()
        for a, s in zip(arr, species):
            a.inertia[:] = s["inertia"]
            a.mass, a.dipole, a.charge = s["mass"], s["dipole"], s["charge"]
            a.nmols, a.rdof, a.framework = s["nmols"], s["rdof"], s["framework"]
            a.name = s["name"].encode()[:L_SPEC - 1]
        self._species = arr
        self._title = title.encode()
        info = _lib.DumpInfo(self._title, istep, interval, level, maxdumps, step * interval, nmols, nmols_r,
                             len(species), arr, int(xdr), dump_init, restart_timestamp)
        self.size = dump_size(level, nmols, nmols_r)
        h = C.c_void_p()
        st = self.L.mdgpu_dump_open(C.byref(h), template.encode(), C.byref(info))
        self._h = h
        if st:
            msg = self.L.mdgpu_dump_errmsg(h).decode()
            self.close()
            raise _lib.MdgpuError(st, msg)

    def append(self, record: np.ndarray) -> str:
        """Writes one record; returns the file it went to."""
        r = np.ascontiguousarray(record, np.float32).reshape(-1)
        if r.size != self.size:
            raise ValueError(f"record has {r.size} floats, the dump level needs {self.size}")
        st = self.L.mdgpu_dump_append(self._h, r.ctypes.data_as(C.POINTER(C.c_float)))
        if st:
            raise _lib.MdgpuError(st, self.L.mdgpu_dump_errmsg(self._h).decode())
        return self.L.mdgpu_dump_filename(self._h).decode()

    def close(self) -> None:
        if self._h:
            self.L.mdgpu_dump_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


@dataclasses.dataclass
class DumpFile:
    xdr: bool
    title: str
    vsn: str
    istep: int
    dump_interval: int
    dump_level: int
    maxdumps: int
    ndumps: int
    dump_size: int
    timestamp: int
    dump_init: int
    restart_timestamp: int
    sysinfo_size: int
    deltat: float
    nmols: int
    nmols_r: int
    species: List[dict]
    records: np.ndarray           # [ndumps, dump_size] float32
    raw_header: bytes             # the header and sysinfo bytes as stored


def _cstr(b: bytes) -> str:
    return b.split(b"\0", 1)[0].decode("latin-1")


def read_dump(path: str) -> DumpFile:
    """One dump file, native (LP64 little-endian) or XDR, as the reference's
    read_dump_header decides (XDR when the version carries "(XDR)")."""
    with open(path, "rb") as f:
        data = f.read()
    h = _HDR_XDR.unpack_from(data, 0)
    xdr = b"(XDR)" in h[1]
    if not xdr:
        h = _HDR_NATIVE.unpack_from(data, 0)
    hs, ss, ms = (_HDR_XDR, _SYS_XDR, _MOL_XDR) if xdr else (_HDR_NATIVE, _SYS_NATIVE, _MOL_NATIVE)
    (title, vsn, istep, interval, level, maxd, nd, size, ts, init, rts, sysz) = h
    o = hs.size
    deltat, nmols, nmols_r, nspec = ss.unpack_from(data, o)
    o += ss.size
    species = []
    for _ in range(nspec):
        v = ms.unpack_from(data, o)
        o += ms.size
        species.append(dict(inertia=list(v[0:3]), mass=v[3], dipole=v[4], charge=v[5], nmols=v[6], rdof=v[7],
                            framework=v[8], name=_cstr(v[9])))
    rec = np.frombuffer(data, dtype=">f4" if xdr else "<f4", count=nd * size, offset=o).astype(np.float32)
    return DumpFile(xdr, _cstr(title), _cstr(vsn), istep, interval, level, maxd, nd, size, ts, init, rts, sysz,
                    deltat, nmols, nmols_r, species, rec.reshape(nd, size), data[:o])
