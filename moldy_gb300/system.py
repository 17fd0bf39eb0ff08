"""System descriptions for the force path, in Moldy's program units.

A :class:`System` carries exactly what Moldy's ``force_calc`` and ``ewald``
read (src/force.c:1108-1320, src/ewald.c:280-589): the unit-cell matrix ``h``
(upper triangular, Å), the species table (sites per molecule, molecule count,
framework flag, site identifiers, principal-frame site coordinates), the
potential-parameter table ``potpar[max_id*max_id][8]`` indexed
``[id_i*max_id + id_j]`` (src/force.c:1202), per-site charges, the
PBC-wrapped site coordinates ``site[3][nsites]`` and the fractional centres of
mass used for molecular-cutoff binning (src/force.c:474-484).

Units follow src/defs.h:213-236: length Å, mass amu, time ps, energy
amu·Å²/ps² (``CONV_E`` kJ/mol per unit) and charge such that Coulomb's law is
q_i q_j / r (``CONV_Q`` elementary charges per unit).

The generators below build the seeded synthetic workloads the force path is
measured on (argon, rigid 4-site water, rock salt).  Each is a plain function
of its size and seed; there is no dataset behind them.
"""
from __future__ import annotations

import dataclasses
import math
import struct
from typing import List, Optional

import numpy as np

# --- unit constants (src/defs.h:201-236, CODATA 1986 values) ---------------
_AVOGAD = 6.0221367e23
_AMU = 1.6605402e-27
_ELCHG = 1.60217733e-19
_ROOT_4_PI_EPS = 1.05482230112e-05
_RTAMU = 4.07497263794495e-14
_EUNIT = _AMU * (1.0e-10 / 1.0e-12) ** 2
#: kJ/mol per program energy unit (src/defs.h:229)
CONV_E = 0.001 * _AVOGAD * _EUNIT
_QUNIT = _RTAMU * 1.0e-3 * _ROOT_4_PI_EPS
#: elementary charges per program charge unit (src/defs.h:235)
CONV_Q = _QUNIT / _ELCHG
PI = 3.14159265358979323846

#: potential type indices, in the order of src/kernel.c:61-68
LJPOT, E6POT, MCYPOT, GENPOT, HIWPOT, RSRVD, MORPOT = 0, 1, 2, 3, 4, 5, 6
#: number of parameters of each potential type (src/kernel.c:61-68)
POT_NPAR = {LJPOT: 2, E6POT: 3, MCYPOT: 4, GENPOT: 6, HIWPOT: 3, MORPOT: 7}
NPOTP = 8  # src/defs.h:144


@dataclasses.dataclass
class Species:
    """One molecular species (the fields of spec_mt the force path reads,
    src/structs.h:121-145)."""
    name: str
    nmols: int
    site_id: np.ndarray          # [nsites] int
    p_f_sites: np.ndarray        # [nsites, 3] principal-frame coordinates, Å
    framework: bool = False

    @property
    def nsites(self) -> int:
        return int(len(self.site_id))


@dataclasses.dataclass
class Control:
    """The control-file keys on the force path (src/startup.c:143-202)."""
    cutoff: float
    alpha: float                 # <= 0: no Ewald (alpha < 0: no Coulomb)
    k_cutoff: float = 0.0
    subcell: float = 0.0         # 0: cutoff/5 (src/force.c:1153)
    strict_cutoff: bool = False
    molpbc: bool = False


@dataclasses.dataclass
class System:
    """Everything ``force_calc``/``ewald`` consume for one configuration."""
    h: np.ndarray                # [3, 3] upper-triangular cell matrix, Å
    species: List[Species]
    ptype: int
    potpar: np.ndarray           # [max_id*max_id, 8] program units
    site_charge: np.ndarray      # [max_id] charge per site identifier
    site: np.ndarray             # [3, nsites] wrapped coordinates, Å
    c_of_m: np.ndarray           # [nmols, 3] fractional centres of mass
    control: Control
    name: str = "system"
    site_mass: Optional[np.ndarray] = None   # [max_id] mass per site identifier, amu
    quat: Optional[np.ndarray] = None        # [nmols_r, 4] orientations of rotating molecules

    @property
    def max_id(self) -> int:
        return int(len(self.site_charge))

    @property
    def nsites(self) -> int:
        return int(sum(s.nsites * s.nmols for s in self.species))

    @property
    def nmols(self) -> int:
        return int(sum(s.nmols for s in self.species))

    @property
    def n_potpar(self) -> int:
        return POT_NPAR[self.ptype]

    def site_ids(self) -> np.ndarray:
        """Expanded per-site identifier array (src/force.c:1184-1190)."""
        return np.concatenate([np.tile(s.site_id, s.nmols) for s in self.species]).astype(np.int32)

    def chg(self) -> np.ndarray:
        """Per-site charges, built as eval_forces does (src/accel.c:480-484)."""
        return self.site_charge[self.site_ids()].astype(np.float64)

    def molmap(self) -> np.ndarray:
        """Molecule index of every site (src/force.c:1175-1182)."""
        return np.concatenate([
            np.repeat(np.arange(s.nmols), s.nsites) + off
            for s, off in zip(self.species, np.cumsum([0] + [s.nmols for s in self.species])[:-1])
        ]).astype(np.int32)

    def volume(self) -> float:
        return float(np.linalg.det(self.h))

    def with_sites(self, site: np.ndarray, c_of_m: Optional[np.ndarray] = None) -> "System":
        return dataclasses.replace(self, site=np.ascontiguousarray(site, dtype=np.float64),
                                   c_of_m=self.c_of_m if c_of_m is None else c_of_m)


# --------------------------------------------------------------------------
# geometry helpers
# --------------------------------------------------------------------------
def _wrap_sites(h: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Put every site into the cell, s -> s - floor(s + 1/2), as make_sites does
    for site-based periodic boundaries (src/algorith.c:201-210)."""
    hinv = np.linalg.inv(h)
    s = hinv @ x
    t = np.floor(s + 0.5)
    return x - h @ t


def _random_quaternions(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random rotations with the distribution random_quat uses
    (src/startup.c:263-280): q0 = sqrt(u), axis uniform on the sphere."""
    phi = 2.0 * PI * rng.random(n)
    cos_t = 1.0 - 2.0 * rng.random(n)
    sin_t = np.sqrt(1.0 - cos_t ** 2)
    q0 = np.sqrt(rng.random(n))
    st2 = np.sqrt(1.0 - q0 ** 2)
    return np.stack([q0, st2 * sin_t * np.sin(phi), st2 * sin_t * np.cos(phi), st2 * cos_t], axis=1)


def _rotation_matrices(q: np.ndarray) -> np.ndarray:
    """Rotation matrices of unit quaternions (principal -> lab frame)."""
    w, x, y, z = q.T
    R = np.empty((len(q), 3, 3))
    R[:, 0, 0] = w * w + x * x - y * y - z * z
    R[:, 0, 1] = 2 * (x * y - w * z)
    R[:, 0, 2] = 2 * (x * z + w * y)
    R[:, 1, 0] = 2 * (x * y + w * z)
    R[:, 1, 1] = w * w - x * x + y * y - z * z
    R[:, 1, 2] = 2 * (y * z - w * x)
    R[:, 2, 0] = 2 * (x * z - w * y)
    R[:, 2, 1] = 2 * (y * z + w * x)
    R[:, 2, 2] = w * w - x * x - y * y + z * z
    return R


def _frac_lattice(n: int) -> np.ndarray:
    """Simple-cubic lattice of n^3 fractional points in [-1/2, 1/2)."""
    g = (np.arange(n) + 0.5) / n - 0.5
    return np.stack(np.meshgrid(g, g, g, indexing="ij"), axis=-1).reshape(-1, 3)


def _potpar(max_id: int) -> np.ndarray:
    return np.zeros((max_id * max_id, NPOTP), dtype=np.float64)


def _set_pot(potpar: np.ndarray, max_id: int, i: int, j: int, params) -> None:
    """Store a pair potential symmetrically, as read_sysdef does
    (src/input.c:344-345)."""
    p = np.zeros(NPOTP)
    p[:len(params)] = params
    potpar[i + j * max_id] = p
    potpar[j + i * max_id] = p


def ewald_k_cutoff(alpha: float, accuracy: float = 1.0e-5) -> float:
    """k_c = 2 alpha sqrt(-ln accuracy) (src/startup.c:760-762)."""
    return 2.0 * alpha * math.sqrt(-math.log(accuracy))


# --------------------------------------------------------------------------
# workloads
# --------------------------------------------------------------------------
def argon_fcc(ncell: int = 5, density: float = 0.0213, displacement: float = 0.1,
              seed: int = 1, cutoff: float = 8.5, subcell: float = 2.0,
              strict: bool = True) -> System:
    """Lennard-Jones argon on an fcc lattice (4*ncell^3 atoms), no charges.

    epsilon 0.996 kJ/mol and sigma 3.405 Å give Moldy's p0 = 4 epsilon
    (src/kernel.c:46 has no factor 4).  Atoms get seeded Gaussian
    displacements of ``displacement`` Å rms so that per-atom forces are not
    zero by symmetry.
    """
    rng = np.random.default_rng(seed)
    natoms = 4 * ncell ** 3
    L = (natoms / density) ** (1.0 / 3.0)
    h = np.diag([L, L, L])
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.arange(ncell)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), axis=-1).reshape(-1, 3)
    frac = ((cells[:, None, :] + basis[None] + 0.25) / ncell).reshape(-1, 3) - 0.5
    x = h @ frac.T + rng.normal(0.0, displacement / math.sqrt(3.0), size=(3, natoms))
    x = _wrap_sites(h, x)
    max_id = 2
    potpar = _potpar(max_id)
    _set_pot(potpar, max_id, 1, 1, [4.0 * 0.996 / CONV_E, 3.405])
    spec = Species("Argon", natoms, np.array([1], np.int32), np.zeros((1, 3)))
    c_of_m = (np.linalg.inv(h) @ x).T
    return System(h=h, species=[spec], ptype=LJPOT, potpar=potpar,
                  site_charge=np.zeros(max_id), site=x, c_of_m=c_of_m,
                  control=Control(cutoff=cutoff, alpha=-1.0, subcell=subcell, strict_cutoff=strict),
                  name=f"argon{natoms}", site_mass=np.array([0.0, 39.948]))


def tip4p_geometry():
    """4-site water: O at the origin, H at (+-0.7570, 0, -0.5859), M 0.15 Å
    along the bisector (O-H 0.9572 Å, HOH 104.52°), shifted to the centre of
    mass (masses O 16, H 1, M 0)."""
    half = math.radians(104.52) / 2.0
    hx, hz = 0.9572 * math.sin(half), -0.9572 * math.cos(half)
    sites = np.array([[0.0, 0.0, 0.0], [hx, 0.0, hz], [-hx, 0.0, hz], [0.0, 0.0, -0.15]])
    masses = np.array([16.0, 1.0, 1.0, 0.0])
    com = (masses[:, None] * sites).sum(0) / masses.sum()
    return sites - com, masses


def water(nside: int = 8, density_gcc: float = 1.0, seed: int = 2, alpha: float = 0.3,
          cutoff: float = 9.0, accuracy: float = 1.0e-5, subcell: float = 0.0,
          strict: bool = False, molpbc: bool = False, model: str = "tip4p") -> System:
    """Rigid 4-site TIP4P-like water, nside^3 molecules on a cubic lattice
    with seeded uniform-random orientations.

    Charges H +0.52 e, M -1.04 e, O 0; LJ on O-O only with epsilon
    0.6485 kJ/mol, sigma 3.154 Å (p0 = 4 epsilon).  The k-space cutoff is set
    for ``accuracy`` as init_cutoffs does (src/startup.c:760-762).
    ``model="mcy"`` swaps the O-O LJ term for an MCY-form O-O/O-H/H-H set so
    that the MCY kernel is exercised on the same geometry.
    """
    rng = np.random.default_rng(seed)
    nmols = nside ** 3
    mass = 18.015
    vol = nmols * mass / (density_gcc * 0.60221367)   # 1 g/cm^3 = 0.6022 amu/Å^3
    L = vol ** (1.0 / 3.0)
    h = np.diag([L, L, L])
    pf, _ = tip4p_geometry()
    com_frac = _frac_lattice(nside)
    q = _random_quaternions(rng, nmols)
    R = _rotation_matrices(q)
    com = (h @ com_frac.T).T
    x = (com[:, None, :] + np.einsum("mij,sj->msi", R, pf)).reshape(-1, 3).T
    x = _wrap_sites(h, x.copy())
    max_id = 4
    potpar = _potpar(max_id)
    if model == "tip4p":
        ptype = LJPOT
        _set_pot(potpar, max_id, 1, 1, [4.0 * 0.6485 / CONV_E, 3.154])
    elif model == "mcy":
        ptype = MCYPOT
        # U = p0 exp(-p1 r) - p2 exp(-p3 r), MCY-like magnitudes (kJ/mol, 1/Å)
        _set_pot(potpar, max_id, 1, 1, [1.088e6 / CONV_E, 5.153, 1.455e3 / CONV_E, 2.961])
        _set_pot(potpar, max_id, 1, 2, [2.733e3 / CONV_E, 2.960, 7.3e2 / CONV_E, 2.233])
        _set_pot(potpar, max_id, 2, 2, [6.667e2 / CONV_E, 2.760, 0.0, 0.0])
    else:
        raise ValueError(model)
    site_charge = np.array([0.0, 0.0, 0.52, -1.04]) / CONV_Q
    spec = Species("Water", nmols, np.array([1, 2, 2, 3], np.int32), pf)
    k_c = ewald_k_cutoff(alpha, accuracy) if alpha > 0 else 0.0
    return System(h=h, species=[spec], ptype=ptype, potpar=potpar, site_charge=site_charge,
                  site=x, c_of_m=com_frac.copy(),
                  control=Control(cutoff=cutoff, alpha=alpha, k_cutoff=k_c, subcell=subcell,
                                  strict_cutoff=strict, molpbc=molpbc),
                  name=f"water{4 * nmols}", site_mass=np.array([0.0, 16.0, 1.0, 0.0]), quat=q)


def water_on_framework(nside: int = 7, nlayers: int = 5, nwall: int = 8, spacing: float = 3.1,
                       seed: int = 6, alpha: float = 0.3, cutoff: float = 9.0, accuracy: float = 1.0e-5,
                       wall_charge: float = 0.4, strict: bool = False) -> System:
    """Rigid water over a charged framework: a cubic box of side
    nside*spacing; a framework molecule of nwall^2 sites on a square grid in
    the plane z = 0 with charges +-``wall_charge`` e in a checkerboard
    (neutral), mass 28 each; nside^2 * nlayers TIP4P-like molecules on a
    lattice between z = 3.6 Å and the periodic image of the wall, seeded
    random orientations.  LJ O-O as in :func:`water`, O-wall epsilon
    0.5 kJ/mol, sigma 3.2 Å; framework-framework pairs are excluded by the
    force path, as the reference excludes them.  Species order: water, then
    the framework (frameworks last, src/input.c:95-117)."""
    rng = np.random.default_rng(seed)
    L = nside * spacing
    if 3.6 + (nlayers - 1) * spacing > L - 3.6:
        raise ValueError("the water layers do not fit between the wall and its image")
    h = np.diag([L, L, L])
    pf, _ = tip4p_geometry()
    g = (np.arange(nside) + 0.5) / nside - 0.5
    zl = (3.6 + spacing * np.arange(nlayers)) / L
    com_frac = np.stack(np.meshgrid(g, g, zl, indexing="ij"), axis=-1).reshape(-1, 3)
    com_frac[:, 2] -= np.floor(com_frac[:, 2] + 0.5)
    nw = len(com_frac)
    q = _random_quaternions(rng, nw)
    R = _rotation_matrices(q)
    xw = ((h @ com_frac.T).T[:, None, :] + np.einsum("mij,sj->msi", R, pf)).reshape(-1, 3)
    # the framework: one molecule; its sites relative to its centre of mass
    gw = (np.arange(nwall) + 0.25) / nwall - 0.5
    wx, wy = np.meshgrid(gw, gw, indexing="ij")
    wall = np.stack([wx.ravel() * L, wy.ravel() * L, np.zeros(nwall * nwall)], axis=1)
    sign = ((np.arange(nwall)[:, None] + np.arange(nwall)[None, :]) % 2).ravel()
    wcom = wall.mean(0)
    wall_pf = wall - wcom
    x = np.concatenate([xw, wall]).T
    x = _wrap_sites(h, x.copy())
    max_id = 6
    potpar = _potpar(max_id)
    _set_pot(potpar, max_id, 1, 1, [4.0 * 0.6485 / CONV_E, 3.154])
    for wid in (4, 5):
        _set_pot(potpar, max_id, 1, wid, [4.0 * 0.5 / CONV_E, 3.2])
    site_charge = np.array([0.0, 0.0, 0.52, -1.04, wall_charge, -wall_charge]) / CONV_Q
    spec_w = Species("Water", nw, np.array([1, 2, 2, 3], np.int32), pf)
    spec_f = Species("Wall", 1, np.where(sign == 0, 4, 5).astype(np.int32), wall_pf, framework=True)
    c_of_m = np.concatenate([com_frac, (np.linalg.inv(h) @ wcom)[None, :]])
    return System(h=h, species=[spec_w, spec_f], ptype=LJPOT, potpar=potpar, site_charge=site_charge,
                  site=x, c_of_m=c_of_m,
                  control=Control(cutoff=cutoff, alpha=alpha, k_cutoff=ewald_k_cutoff(alpha, accuracy),
                                  strict_cutoff=strict),
                  name=f"waterwall{4 * nw + nwall * nwall}",
                  site_mass=np.array([0.0, 16.0, 1.0, 0.0, 28.0, 28.0]), quat=q)


def rock_salt(ncell: int = 16, a: float = 5.64, displacement: float = 0.1, seed: int = 3,
              alpha: float = 0.35, cutoff: float = 10.0, accuracy: float = 1.0e-5,
              k_cutoff: Optional[float] = None) -> System:
    """NaCl-structure ionic solid, 8*ncell^3 ions with charges +-1 e.

    Born-Mayer-Huggins/Buckingham in Moldy's 6-exp form
    U = -p0/r^6 + p1 exp(-p2 r) (src/kernel.c:47): the +- pair is
    (0, 1.2e5 kJ/mol, 1/0.317 Å^-1), the -- pair (7000 kJ/mol Å^6, 0, 0), the
    ++ pair zero.  Ions get seeded Gaussian displacements of
    ``displacement`` Å rms.
    """
    rng = np.random.default_rng(seed)
    L = ncell * a
    h = np.diag([L, L, L])
    fcc = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.arange(ncell)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), axis=-1).reshape(-1, 3)
    na = ((cells[:, None, :] + fcc[None] + 0.125) / ncell).reshape(-1, 3) - 0.5
    cl = ((cells[:, None, :] + fcc[None] + np.array([0.5, 0, 0]) + 0.125) / ncell).reshape(-1, 3) - 0.5
    n = len(na)
    xna = h @ na.T + rng.normal(0.0, displacement / math.sqrt(3.0), size=(3, n))
    xcl = h @ cl.T + rng.normal(0.0, displacement / math.sqrt(3.0), size=(3, n))
    x = _wrap_sites(h, np.concatenate([xna, xcl], axis=1))
    max_id = 3
    potpar = _potpar(max_id)
    _set_pot(potpar, max_id, 1, 2, [0.0, 1.2e5 / CONV_E, 1.0 / 0.317])
    _set_pot(potpar, max_id, 2, 2, [7000.0 / CONV_E, 0.0, 0.0])
    site_charge = np.array([0.0, 1.0, -1.0]) / CONV_Q
    species = [Species("Na", n, np.array([1], np.int32), np.zeros((1, 3))),
               Species("Cl", n, np.array([2], np.int32), np.zeros((1, 3)))]
    k_c = ewald_k_cutoff(alpha, accuracy) if k_cutoff is None else k_cutoff
    c_of_m = (np.linalg.inv(h) @ x).T
    return System(h=h, species=species, ptype=E6POT, potpar=potpar, site_charge=site_charge,
                  site=x, c_of_m=c_of_m,
                  control=Control(cutoff=cutoff, alpha=alpha, k_cutoff=k_c),
                  name=f"rocksalt{2 * n}", site_mass=np.array([0.0, 22.98977, 35.453]))


def generic_ions(ptype: int, n: int = 256, L: float = 20.0, seed: int = 4, alpha: float = 0.35,
                 cutoff: float = 8.0) -> System:
    """Small random two-species ionic system for the generic, HIW and Morse
    kernels (src/kernel.c:264-354).  Ions sit on a jittered lattice so that no
    pair comes closer than about 1.7 Å."""
    rng = np.random.default_rng(seed)
    side = int(round(n ** (1.0 / 3.0)))
    n = side ** 3
    h = np.diag([L, L, L])
    frac = _frac_lattice(side) + rng.normal(0.0, 0.05 / side, size=(n, 3))
    x = _wrap_sites(h, h @ frac.T)
    max_id = 3
    potpar = _potpar(max_id)
    E = 1.0 / CONV_E
    if ptype == GENPOT:
        _set_pot(potpar, max_id, 1, 1, [5.0e4 * E, 3.2, 1.0e3 * E, 10.0 * E, 20.0 * E, 30.0 * E])
        _set_pot(potpar, max_id, 1, 2, [9.0e4 * E, 3.4, 2.0e3 * E, 15.0 * E, 40.0 * E, 20.0 * E])
        _set_pot(potpar, max_id, 2, 2, [7.0e4 * E, 3.0, 1.5e3 * E, 5.0 * E, 60.0 * E, 25.0 * E])
    elif ptype == HIWPOT:
        _set_pot(potpar, max_id, 1, 1, [-50.0 * E, -300.0 * E, 4.0e5 * E])
        _set_pot(potpar, max_id, 1, 2, [-80.0 * E, -500.0 * E, 9.0e5 * E])
        _set_pot(potpar, max_id, 2, 2, [-60.0 * E, -400.0 * E, 6.0e5 * E])
    elif ptype == MORPOT:
        _set_pot(potpar, max_id, 1, 1, [20.0 * E, 3.0, 3.5, 300.0 * E, 5.0 * E, 1.8, 2.6])
        _set_pot(potpar, max_id, 1, 2, [25.0 * E, 3.2, 3.3, 500.0 * E, 8.0 * E, 1.6, 2.5])
        _set_pot(potpar, max_id, 2, 2, [30.0 * E, 3.4, 3.1, 700.0 * E, 6.0 * E, 1.7, 2.7])
    elif ptype in (LJPOT, E6POT, MCYPOT):
        raise ValueError("use the named workloads for LJ, 6-exp and MCY")
    else:
        raise ValueError(ptype)
    half = n // 2
    site_charge = np.array([0.0, 0.8, -0.8]) / CONV_Q
    species = [Species("A", half, np.array([1], np.int32), np.zeros((1, 3))),
               Species("B", n - half, np.array([2], np.int32), np.zeros((1, 3)))]
    c_of_m = (np.linalg.inv(h) @ x).T
    return System(h=h, species=species, ptype=ptype, potpar=potpar, site_charge=site_charge,
                  site=x, c_of_m=c_of_m,
                  control=Control(cutoff=cutoff, alpha=alpha, k_cutoff=ewald_k_cutoff(alpha)),
                  name=f"ptype{ptype}_{n}")


# --------------------------------------------------------------------------
# binary exchange format (read by the reference harness under oracle/)
# --------------------------------------------------------------------------
MDSYS_MAGIC = b"MDSYS1\0\0"


def write_mdsys(path: str, sysm: System, want_pairs: bool = False) -> None:
    """Write ``sysm`` in the flat little-endian layout the oracle harness
    reads: header ints, control doubles, h, species blocks, potpar, site
    charges, site coordinates (SoA) and fractional centres of mass."""
    c = sysm.control
    with open(path, "wb") as f:
        f.write(MDSYS_MAGIC)
        f.write(struct.pack("<8i", sysm.nsites, sysm.nmols, len(sysm.species), sysm.max_id,
                            sysm.ptype, int(c.strict_cutoff), int(c.molpbc), int(want_pairs)))
        f.write(struct.pack("<4d", c.cutoff, c.subcell, c.alpha, c.k_cutoff))
        f.write(np.ascontiguousarray(sysm.h, dtype="<f8").tobytes())
        for s in sysm.species:
            f.write(struct.pack("<4i", s.nsites, s.nmols, int(s.framework), 0))
            f.write(np.ascontiguousarray(s.site_id, dtype="<i4").tobytes())
            f.write(np.ascontiguousarray(s.p_f_sites, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(sysm.potpar, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(sysm.site_charge, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(sysm.site, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(sysm.c_of_m, dtype="<f8").tobytes())


def read_mdsys(path: str, name: str = "mdsys") -> System:
    """Inverse of :func:`write_mdsys`."""
    raw = open(path, "rb").read()
    if raw[:6] != MDSYS_MAGIC[:6]:
        raise ValueError(f"{path}: not an MDSYS1 file")
    off = 8
    nsites, nmols, nspecies, max_id, ptype, strict, molpbc, _ = struct.unpack_from("<8i", raw, off)
    off += 32
    cutoff, subcell, alpha, k_cutoff = struct.unpack_from("<4d", raw, off)
    off += 32
    h = np.frombuffer(raw, "<f8", 9, off).reshape(3, 3).copy()
    off += 72
    species = []
    for s in range(nspecies):
        ns, nm, fw, _ = struct.unpack_from("<4i", raw, off)
        off += 16
        ids = np.frombuffer(raw, "<i4", ns, off).copy()
        off += 4 * ns
        pf = np.frombuffer(raw, "<f8", 3 * ns, off).reshape(ns, 3).copy()
        off += 24 * ns
        species.append(Species(f"s{s}", nm, ids, pf, bool(fw)))
    potpar = np.frombuffer(raw, "<f8", max_id * max_id * NPOTP, off).reshape(-1, NPOTP).copy()
    off += 8 * max_id * max_id * NPOTP
    site_charge = np.frombuffer(raw, "<f8", max_id, off).copy()
    off += 8 * max_id
    site = np.frombuffer(raw, "<f8", 3 * nsites, off).reshape(3, nsites).copy()
    off += 24 * nsites
    c_of_m = np.frombuffer(raw, "<f8", 3 * nmols, off).reshape(nmols, 3).copy()
    return System(h=h, species=species, ptype=ptype, potpar=potpar, site_charge=site_charge,
                  site=site, c_of_m=c_of_m,
                  control=Control(cutoff=cutoff, alpha=alpha, k_cutoff=k_cutoff, subcell=subcell,
                                  strict_cutoff=bool(strict), molpbc=bool(molpbc)), name=name)


def save_npz(path: str, sysm: System, **extra) -> None:
    """Store a System (and any extra arrays) in one compressed .npz."""
    c = sysm.control
    d = dict(h=sysm.h, ptype=sysm.ptype, potpar=sysm.potpar, site_charge=sysm.site_charge,
             site=sysm.site, c_of_m=sysm.c_of_m, name=sysm.name,
             control=np.array([c.cutoff, c.alpha, c.k_cutoff, c.subcell, float(c.strict_cutoff),
                               float(c.molpbc)]),
             spec_nmols=np.array([s.nmols for s in sysm.species]),
             spec_nsites=np.array([s.nsites for s in sysm.species]),
             spec_fw=np.array([int(s.framework) for s in sysm.species]),
             spec_ids=np.concatenate([s.site_id for s in sysm.species]),
             spec_pf=np.concatenate([s.p_f_sites for s in sysm.species]))
    if sysm.site_mass is not None:
        d["site_mass"] = sysm.site_mass
    if sysm.quat is not None:
        d["quat"] = sysm.quat
    d.update(extra)
    np.savez_compressed(path, **d)


def load_npz(path: str):
    """Returns (System, dict of all arrays in the file)."""
    z = dict(np.load(path, allow_pickle=False))
    species, o = [], 0
    for k, (nm, ns, fw) in enumerate(zip(z["spec_nmols"], z["spec_nsites"], z["spec_fw"])):
        species.append(Species(f"s{k}", int(nm), z["spec_ids"][o:o + ns].astype(np.int32),
                               z["spec_pf"][o:o + ns], bool(fw)))
        o += ns
    c = z["control"]
    sysm = System(h=z["h"], species=species, ptype=int(z["ptype"]), potpar=z["potpar"],
                  site_charge=z["site_charge"], site=z["site"], c_of_m=z["c_of_m"],
                  control=Control(cutoff=float(c[0]), alpha=float(c[1]), k_cutoff=float(c[2]),
                                  subcell=float(c[3]), strict_cutoff=bool(c[4]), molpbc=bool(c[5])),
                  name=str(z["name"]), site_mass=z.get("site_mass"), quat=z.get("quat"))
    return sysm, z
