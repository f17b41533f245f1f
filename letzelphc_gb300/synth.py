"""Seeded synthetic inputs for the per-q electron-phonon matrix-element stage.

LetzElPhC reads its inputs from a yambo SAVE directory and a QE ph_save
directory (src/io/get_save_data.c:51, src/io/qe/get_dvscf_dyn_qe.c:15).  None
of those real systems exist here, so every workload is a seeded synthetic
system with the shapes, sizes and value distributions of the named
configurations.  All arrays use the reference's own conventions
(src/common/dtypes.h:80-266):

* ``alat``  (3,3): lattice vectors as COLUMNS, a_i = alat[:, i] (bohr).
* ``blat``  (3,3): reciprocal vectors as columns, INCLUDING 2*pi, computed as
  ``reciprocal_vecs`` does with the truncated pi (src/common/numerical_func.c:280-298).
* k-points and G-vectors: cartesian, in units without 2*pi (k_cart = A^-T k_crys).
* ``sym_R`` (nsym,3,3) cartesian rotations acting as v' = R v; ``sym_tau``
  (nsym,3) cartesian fractional translations; time-reversal copies carry
  (-R, -tau) and come second (src/io/get_save_data.c:264-302).
* ``kmap`` (nk_BZ,2) = (iBZ k, symmetry), built the way ``bz_expand`` builds
  it (src/symmetries/BZ_expand.c:11-97).
* wavefunctions (nspin, nbnd, nspinor, npw) complex, Gram-Schmidt
  orthonormalised per k; dV_scf (nmodes, nmag, Nx, Ny, Nz) complex;
  eigVec (nmodes, 3*natom) complex unitary.
* KB data: PP_table (nltimesj, ntype, 3) rows (l+1, 2j, 1), Fsign
  (nltimesj, ntype), Fk per k (nltimesj, ntype, npw), fCoeff per
  (lidx, itype) of shape (2l+1, 2l+1, nspinor, nspinor) or None.
"""
from __future__ import annotations

import itertools
import math
import struct
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

ELPH_PI = 3.1415927          # src/common/constants.h:11 (also in the double build)
ELPH_SQRT2 = 1.4142136       # src/common/constants.h:12
ELPH_EPS = 1e-5              # src/common/constants.h:9
ELPH_E2 = 2.0                # src/common/constants.h:13


def reciprocal_vecs(alat: np.ndarray) -> np.ndarray:
    """b_i (columns, with the truncated 2*pi) from the cofactors of alat,
    following src/common/numerical_func.c:280-298."""
    a = alat.reshape(9)
    det = (a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6])
           + a[2] * (a[7] * a[3] - a[4] * a[6]))
    f = 2 * ELPH_PI / det
    b = np.empty(9)
    b[0] = (a[4] * a[8] - a[7] * a[5]) * f
    b[1] = (a[5] * a[6] - a[3] * a[8]) * f
    b[2] = (a[3] * a[7] - a[6] * a[4]) * f
    b[3] = (a[2] * a[7] - a[1] * a[8]) * f
    b[4] = (a[0] * a[8] - a[2] * a[6]) * f
    b[5] = (a[1] * a[6] - a[0] * a[7]) * f
    b[6] = (a[1] * a[5] - a[2] * a[4]) * f
    b[7] = (a[2] * a[3] - a[0] * a[5]) * f
    b[8] = (a[0] * a[4] - a[1] * a[3]) * f
    return b.reshape(3, 3)


def find_kidx_in_list(klist: np.ndarray, kpt: np.ndarray) -> int:
    """Periodic search with tolerance ELPH_EPS (src/common/numerical_func.c:471-497)."""
    if len(klist) == 0:
        return -1
    d = klist - kpt[None, :]
    d = d - np.rint(d)
    s = np.sqrt((d * d).sum(axis=1))
    hit = np.nonzero(s < ELPH_EPS)[0]
    return int(hit[0]) if len(hit) else -1


# --------------------------------------------------------------------------
# crystal structures
# --------------------------------------------------------------------------

def _structure(kind: str, a: float):
    """Return (alat columns, fractional positions, types, dimension char)."""
    if kind == "diamond":        # fcc Si-like, atoms at 0 and a/4(1,1,1)
        A = 0.5 * a * np.array([[0, 1, 1], [1, 0, 1], [1, 1, 0]], float)
        cart = np.array([[0, 0, 0], [0.25 * a] * 3])
        frac = np.linalg.solve(A, cart.T).T
        return A, frac, np.array([0, 0]), "3"
    if kind == "zincblende":     # same cell, two species: T_d, no inversion
        A, frac, _, d = _structure("diamond", a)
        return A, frac, np.array([0, 1]), d
    if kind == "l12":            # simple cubic, 4 atoms (Cu3Au type), origin shifted
        A = a * np.eye(3)
        frac = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
        frac = frac + np.array([0.0625, 0.125, 0.1875])   # generic origin -> tau != 0
        return A, frac, np.array([0, 1, 1, 1]), "3"
    if kind == "hex2d":          # 3-atom MX2-like slab, c/a = 6
        c = 6.0 * a
        A = np.array([[a, -0.5 * a, 0], [0, math.sqrt(3) / 2 * a, 0], [0, 0, c]])
        frac = np.array([[1 / 3, 2 / 3, 0.5], [2 / 3, 1 / 3, 0.5 + 0.05], [2 / 3, 1 / 3, 0.5 - 0.05]])
        return A, frac, np.array([0, 1, 1]), "2"
    if kind == "rocksalt8":      # simple cubic 8-atom rock-salt cell
        A = a * np.eye(3)
        f0 = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
        frac = np.vstack([f0, f0 + 0.5]) % 1.0
        frac = frac + np.array([0.03125, 0.0625, 0.09375])
        return A, frac, np.array([0, 0, 0, 0, 1, 1, 1, 1]), "3"
    if kind == "sc16":           # simple cubic 16-atom cell (two fcc + two shifted)
        A = a * np.eye(3)
        f0 = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
        frac = np.vstack([f0, f0 + 0.25, f0 + 0.5, f0 + 0.75]) % 1.0
        return A, frac, np.array([0] * 8 + [1] * 8), "3"
    raise ValueError(kind)


def find_symmetries(A: np.ndarray, frac: np.ndarray, types: np.ndarray, timerev: bool):
    """Space-group operations {R|tau} of the structure (cartesian), identity first.

    Rotations are searched as integer matrices W in crystal coordinates with
    entries in {-1,0,1} preserving the metric; tau from mapping atom 0 onto
    every atom of its species."""
    M = A.T @ A
    Ainv = np.linalg.inv(A)
    ops = []
    for ent in itertools.product((-1, 0, 1), repeat=9):
        W = np.array(ent, float).reshape(3, 3)
        if abs(abs(np.linalg.det(W)) - 1) > 1e-8:
            continue
        if np.abs(W.T @ M @ W - M).max() > 1e-6 * np.abs(M).max():
            continue
        for j in np.nonzero(types == types[0])[0]:
            tau = frac[j] - W @ frac[0]
            ok = True
            for i in range(len(frac)):
                xi = W @ frac[i] + tau
                d = frac - xi
                d -= np.rint(d)
                hit = np.nonzero((np.abs(d).max(axis=1) < 1e-8) & (types == types[i]))[0]
                if len(hit) != 1:
                    ok = False
                    break
            if ok:
                tau = tau - np.floor(tau + 1e-9)
                tau[np.abs(tau) < 1e-12] = 0.0
                ops.append((W, tau))
                break
    ops.sort(key=lambda o: (0 if np.allclose(o[0], np.eye(3)) else 1))
    R = np.array([A @ W @ Ainv for W, _ in ops])
    T = np.array([A @ t for _, t in ops])
    R[np.abs(R) < 1e-14] = 0.0
    T[np.abs(T) < 1e-14] = 0.0
    trev = np.zeros(len(ops), bool)
    if timerev:
        R = np.concatenate([R, -R])
        T = np.concatenate([T, -T])
        trev = np.concatenate([trev, np.ones(len(ops), bool)])
    return R, T, trev


def bz_expand(kibz_cart: np.ndarray, sym_R: np.ndarray, alat: np.ndarray):
    """iBZ (cart) -> full BZ (crystal) and kmap, in the order of
    src/symmetries/BZ_expand.c:25-52."""
    kpts = []
    kmap = []
    for ik, k in enumerate(kibz_cart):
        for isym, R in enumerate(sym_R):
            kc = R @ k
            kcrys = alat.T @ kc
            if find_kidx_in_list(np.array(kpts).reshape(-1, 3), kcrys) < 0:
                kpts.append(kcrys)
                kmap.append((ik, isym))
    return np.array(kpts), np.array(kmap, np.int32)


def reduce_grid(kgrid, sym_R, alat):
    """Irreducible points of a Gamma-centred grid (crystal), in grid order."""
    n1, n2, n3 = kgrid
    Ainv_T = np.linalg.inv(alat).T
    pts = []
    for i in range(n1):
        for j in range(n2):
            for l in range(n3):
                pts.append(np.array([i / n1, j / n2, l / n3]))
    pts = np.array(pts)
    pts = pts - np.rint(pts)        # into (-1/2, 1/2]
    covered = np.zeros(len(pts), bool)
    ibz = []
    for ip, k in enumerate(pts):
        if covered[ip]:
            continue
        ibz.append(k)
        kc = Ainv_T @ k
        for R in sym_R:
            kk = alat.T @ (R @ kc)
            idx = find_kidx_in_list(pts, kk)
            if idx >= 0:
                covered[idx] = True
    return np.array(ibz)


# --------------------------------------------------------------------------
# SOC f coefficients (restated from src/nonloc/fcoeff.c:24-283)
# --------------------------------------------------------------------------

def _cmat(m1, m2):
    a1, a2 = abs(m1), abs(m2)
    if a1 != a2:
        return 0.0
    if m1 == 0 and m2 == 0:
        return 1.0
    if m1 == a1 and m2 == a2:
        return (-1.0) ** a1 / ELPH_SQRT2
    if m1 == -a1 and m2 == a2:
        return 1.0 / ELPH_SQRT2
    if m1 == a1 and m2 == -a2:
        return 1j * (-1.0) ** a1 / ELPH_SQRT2
    return -1j / ELPH_SQRT2


def _umat(jp1, down, l, twomj, m2):
    if jp1:
        m = (twomj - 1) // 2
        return _cmat(m, m2) if not down else _cmat(m + 1, m2)
    m = (twomj + 1) // 2
    return _cmat(m - 1, m2) if not down else _cmat(m, m2)


def _cg(jp1, down, l, twomj):
    mj = twomj / 2.0
    if jp1:
        m = mj - 0.5
        return math.sqrt((l + m + 1.0) / (2.0 * l + 1.0)) if not down else math.sqrt((l - m) / (2.0 * l + 1.0))
    m = mj + 0.5
    return math.sqrt((l - m + 1.0) / (2.0 * l + 1.0)) if not down else -math.sqrt((l + m) / (2.0 * l + 1.0))


def f_coeff(l: int, twoj: int, nspinor: int) -> np.ndarray:
    jp1 = twoj == 2 * l + 1
    if not jp1 and twoj != 2 * l - 1:
        raise ValueError("inconsistent j")
    n = 2 * l + 1
    out = np.zeros((n, n, nspinor, nspinor), complex)
    for i1 in range(n):
        for i2 in range(n):
            for s1 in range(nspinor):
                for s2 in range(nspinor):
                    acc = 0j
                    for mj in range(-twoj, twoj + 1, 2):
                        acc += (_cg(jp1, s1, l, mj) * _cg(jp1, s2, l, mj)
                                * _umat(jp1, s1, l, mj, i1 - l) * np.conj(_umat(jp1, s2, l, mj, i2 - l)))
                    out[i1, i2, s1, s2] = acc
    return out


# --------------------------------------------------------------------------
# configurations
# --------------------------------------------------------------------------

CONFIGS: Dict[str, dict] = {
    # 2-atom fcc diamond, 24^3, npw ~400, 4x4x4 k, q=(0.25,0,0), 6 modes, 8 bands
    "c0": dict(kind="diamond", a=10.26, fft=(24, 24, 24), kgrid=(4, 4, 4),
               qpts=[(0.25, 0, 0)], nbnds=8, npw=400, ls=(0, 1), seed=1000),
    # 4-atom cell, 48^3, npw ~2500, 8x8x8 k, 8 q, 12 modes, 32 bands
    "c1": dict(kind="l12", a=7.1, fft=(48, 48, 48), kgrid=(8, 8, 8),
               qpts=[(0, 0, 0), (0.125, 0, 0), (0.25, 0, 0), (0.375, 0, 0), (0.5, 0, 0),
                     (0.125, 0.125, 0), (0.25, 0.25, 0), (0.25, 0.125, 0.125)],
               nbnds=32, npw=2500, ls=(0, 1), seed=1001),
    # 3-atom hexagonal 2D slab, 36x36x216, 12x12x1 k, 64 q, 9 modes, 40 bands, npw 1800-2600
    "c2": dict(kind="hex2d", a=6.0, fft=(36, 36, 216), kgrid=(12, 12, 1),
               qpts="grid64", nbnds=40, npw=(1800, 2600), ls=(0, 1), seed=1002),
    # 8-atom spinor SOC cell, 60^3, npw ~5000, 6x6x6 k, 4 q, 24 modes, 64 bands, l=0..2
    "c3": dict(kind="rocksalt8", a=8.0, fft=(60, 60, 60), kgrid=(6, 6, 6),
               qpts=[(0, 0, 0), (1 / 6, 0, 0), (1 / 3, 0, 0), (1 / 6, 1 / 6, 0)],
               nbnds=64, npw=5000, ls=(0, 1, 2), nspinor=2, nmag=4, soc=True, seed=1003),
    # 16-atom cell, 96^3, npw ~12000, 200 bands, 8x8x8 k, 48 modes, 29 iBZ q
    "c4": dict(kind="sc16", a=10.0, fft=(96, 96, 96), kgrid=(8, 8, 8),
               qpts="ibz", nbnds=200, npw=12000, ls=(0, 1), seed=1004),
}


@dataclass
class System:
    name: str
    alat: np.ndarray
    blat: np.ndarray
    atom_pos: np.ndarray           # (natom,3) cart
    atom_type: np.ndarray          # (natom,) int
    ntype: int
    dimension: str
    sym_R: np.ndarray              # (nsym,3,3)
    sym_tau: np.ndarray            # (nsym,3)
    sym_trev: np.ndarray           # (nsym,) bool
    timerev: int
    kibz: np.ndarray               # (nk_ibz,3) cart
    kbz_crys: np.ndarray           # (nk_bz,3)
    kmap: np.ndarray               # (nk_bz,2)
    fft_dims: tuple
    nspin: int
    nspinor: int
    nmag: int
    nbnds: int
    gvec: List[np.ndarray]         # per iBZ k (npw,3) cart
    miller: List[np.ndarray]       # per iBZ k (npw,3) int
    wfc: List[np.ndarray]          # per iBZ k (nspin,nbnd,nspinor,npw) complex
    Fk: List[np.ndarray]           # per iBZ k (nltimesj,ntype,npw)
    PP_table: np.ndarray           # (nltimesj,ntype,3)
    Fsign: np.ndarray              # (nltimesj,ntype)
    fCoeff: Optional[list]         # [(lidx*ntype+itype)] -> array or None
    lmax: int
    is_soc_present: bool
    qpts: np.ndarray               # (nq,3) crystal
    eigVec: np.ndarray             # (nq, nmodes, nmodes)
    dVscf: np.ndarray              # (nq, nmodes, nmag, Nx, Ny, Nz)
    extra: dict = field(default_factory=dict)
    # local pseudopotential per species (struct local_pseudo): radial mesh,
    # its derivative, V_loc(r) in Ry, valence charge
    loc_r: Optional[list] = None
    loc_rab: Optional[list] = None
    loc_v: Optional[list] = None
    loc_zval: Optional[np.ndarray] = None

    @property
    def natom(self):
        return len(self.atom_type)

    @property
    def nmodes(self):
        return 3 * self.natom

    @property
    def nk_ibz(self):
        return len(self.kibz)

    @property
    def nk_bz(self):
        return len(self.kbz_crys)

    @property
    def nltimesj(self):
        return self.PP_table.shape[0]

    @property
    def npw(self):
        return np.array([len(g) for g in self.gvec])


def _sphere(k_crys, alat, Ainv_T, ecut):
    gc = math.sqrt(ecut)
    lim = [int(math.ceil(np.linalg.norm(alat[:, i]) * gc)) + 2 for i in range(3)]
    rr = [np.arange(-m, m + 1) for m in lim]
    n = np.array(np.meshgrid(*rr, indexing="ij")).reshape(3, -1).T
    kg = (n + k_crys[None, :]) @ Ainv_T.T
    e = (kg * kg).sum(1)
    sel = e <= ecut
    n = n[sel]
    e = e[sel]
    order = np.lexsort((n[:, 2], n[:, 1], n[:, 0], np.round(e, 12)))
    return n[order]


def _ecut_for(npw_target, Ainv_T, nmax):
    # the number of G with |G| <= Gc is ~ (4/3) pi Gc^3 / det(Ainv_T)
    vol = 1.0 / abs(np.linalg.det(Ainv_T))
    gc = (3.0 * npw_target / (4.0 * math.pi * vol)) ** (1.0 / 3.0)
    return gc * gc


def make_system(name: str = "c0", overrides: Optional[dict] = None) -> System:
    """Build the seeded synthetic system of a named configuration.

    ``overrides`` changes any key (e.g. ``nbnds``, ``kgrid``, ``qpts``,
    ``timerev``, ``nspin``...) so tests can derive small variants."""
    cfg = dict(CONFIGS[name.split(":")[0]] if name.split(":")[0] in CONFIGS else {})
    if overrides:
        cfg.update(overrides)
    rng = np.random.default_rng(cfg.get("seed", 1000))
    A, frac, types, dim = _structure(cfg["kind"], cfg["a"])
    timerev = bool(cfg.get("timerev", False))
    sym_R, sym_tau, sym_trev = find_symmetries(A, frac, types, timerev)
    if cfg.get("nsym_max"):
        nkeep = cfg["nsym_max"]
        sym_R, sym_tau, sym_trev = sym_R[:nkeep], sym_tau[:nkeep], sym_trev[:nkeep]
    blat = reciprocal_vecs(A)
    Ainv_T = np.linalg.inv(A).T
    kibz_crys = reduce_grid(cfg["kgrid"], sym_R, A)
    kibz = kibz_crys @ Ainv_T.T
    kbz_crys, kmap = bz_expand(kibz, sym_R, A)
    nkg = int(np.prod(cfg["kgrid"]))
    if len(kbz_crys) != nkg:
        raise RuntimeError(f"bz_expand found {len(kbz_crys)} points, grid has {nkg}")

    nspin = cfg.get("nspin", 1)
    nspinor = cfg.get("nspinor", 1)
    nmag = cfg.get("nmag", 2 if nspin == 2 else 1)
    nb = cfg["nbnds"]
    fft = tuple(cfg["fft"])
    natom = len(types)
    ntype = int(types.max()) + 1
    nmodes = 3 * natom

    # plane-wave spheres
    npw_spec = cfg["npw"]
    nmax = max(fft) // 2
    gvec, miller, wfc, Fk = [], [], [], []
    ls = cfg.get("ls", (0, 1))
    soc = bool(cfg.get("soc", False))
    if soc:
        rows = []
        for l in ls:
            for twoj in ((2 * l + 1,) if l == 0 else (2 * l - 1, 2 * l + 1)):
                rows.append((l, twoj))
    else:
        rows = [(l, 0) for l in ls]
    nltimesj = len(rows)
    PP_table = np.zeros((nltimesj, ntype, 3))
    for il, (l, twoj) in enumerate(rows):
        PP_table[il, :, 0] = l + 1
        PP_table[il, :, 1] = twoj
        PP_table[il, :, 2] = 1
    Fsign = rng.choice([-1.0, 1.0], size=(nltimesj, ntype))
    Fsign[0, :] = 1.0
    famp = rng.uniform(0.5, 1.5, size=(nltimesj, ntype))
    for ik, kc in enumerate(kibz_crys):
        if isinstance(npw_spec, tuple):
            target = rng.uniform(npw_spec[0], npw_spec[1])
        else:
            target = npw_spec
        ecut = _ecut_for(target, Ainv_T, nmax)
        n = _sphere(kc, A, Ainv_T, ecut)
        miller.append(n.astype(np.int32))
        g = n @ Ainv_T.T
        gvec.append(g)
        npw = len(n)
        c = rng.standard_normal((nspin, nb, nspinor * npw)) + 1j * rng.standard_normal((nspin, nb, nspinor * npw))
        for s in range(nspin):
            q, _ = np.linalg.qr(c[s].T)
            c[s] = q.T
        wfc.append(c.reshape(nspin, nb, nspinor, npw))
        kg = np.sqrt((((n + kc[None, :]) @ Ainv_T.T) ** 2).sum(1))
        gc = math.sqrt(ecut)
        F = np.zeros((nltimesj, ntype, npw))
        for il, (l, _) in enumerate(rows):
            for it in range(ntype):
                F[il, it] = famp[il, it] * np.exp(-(kg / (0.5 * gc)) ** 2) * (kg / gc) ** l
        Fk.append(F)
    gcut_dv = math.sqrt(_ecut_for(np.mean([len(m) for m in miller]), Ainv_T, nmax))

    fCoeff = None
    if soc and nspinor == 2:
        fCoeff = []
        for il, (l, twoj) in enumerate(rows):
            for it in range(ntype):
                fCoeff.append(f_coeff(l, twoj, nspinor) if twoj != 0 else None)

    # q points
    qspec = cfg["qpts"]
    if qspec == "grid64":
        g = [np.array([i / cfg["kgrid"][0], j / cfg["kgrid"][1], 0.0]) for i in range(8) for j in range(8)]
        qpts = np.array(g)
    elif qspec == "ibz":
        qpts = reduce_grid(cfg["kgrid"], sym_R, A)
    else:
        qpts = np.array(qspec, float).reshape(-1, 3)
    nq = len(qpts)

    # dV_scf: complex normal in G, Gaussian of width 0.3 G_cut, unnormalised inverse FFT
    Nx, Ny, Nz = fft
    fx = np.fft.fftfreq(Nx, 1.0 / Nx)
    fy = np.fft.fftfreq(Ny, 1.0 / Ny)
    fz = np.fft.fftfreq(Nz, 1.0 / Nz)
    M = np.array(np.meshgrid(fx, fy, fz, indexing="ij")).reshape(3, -1).T
    G2 = ((M @ Ainv_T.T) ** 2).sum(1).reshape(Nx, Ny, Nz)
    gauss = np.exp(-G2 / (2.0 * (0.3 * gcut_dv) ** 2))
    dV = np.empty((nq, nmodes, nmag, Nx, Ny, Nz), complex)
    eig = np.empty((nq, nmodes, nmodes), complex)
    for iq in range(nq):
        z = rng.standard_normal((nmodes, nmag, Nx, Ny, Nz)) + 1j * rng.standard_normal((nmodes, nmag, Nx, Ny, Nz))
        v = np.fft.ifftn(z * gauss, axes=(2, 3, 4)) * (Nx * Ny * Nz)
        v /= np.sqrt(np.mean(np.abs(v) ** 2))
        dV[iq] = v
        e = rng.standard_normal((nmodes, nmodes)) + 1j * rng.standard_normal((nmodes, nmodes))
        eig[iq] = np.linalg.qr(e)[0]

    sysm = System(name=name, alat=A, blat=blat, atom_pos=frac @ A.T, atom_type=types.astype(np.int32),
                  ntype=ntype, dimension=dim, sym_R=sym_R, sym_tau=sym_tau, sym_trev=sym_trev,
                  timerev=int(timerev), kibz=kibz, kbz_crys=kbz_crys, kmap=kmap, fft_dims=fft,
                  nspin=nspin, nspinor=nspinor, nmag=nmag, nbnds=nb, gvec=gvec, miller=miller, wfc=wfc,
                  Fk=Fk, PP_table=PP_table, Fsign=Fsign, fCoeff=fCoeff, lmax=max(ls),
                  is_soc_present=soc, qpts=qpts, eigVec=eig, dVscf=dV)
    local_pseudo(sysm, cfg.get("seed", 1000))
    check_box(sysm)
    return sysm


def local_pseudo(s: System, seed: int):
    """Seeded local pseudopotential of every species (own generator, so the
    rest of the system does not depend on it): a QE-style logarithmic mesh
    r_i = exp(xmin + i dx) / Z, rab_i = r_i dx, out to ~10 bohr, and
    V_loc(r) = -Z e2 erf(r / rc) / r + a exp(-(r / w)^2) (Ry, e2 = 2)."""
    rng = np.random.default_rng(seed + 7919)
    e2 = 2.0
    s.loc_zval = rng.choice([1.0, 3.0, 4.0, 5.0, 6.0], size=s.ntype)
    s.loc_r, s.loc_rab, s.loc_v = [], [], []
    for t in range(s.ntype):
        z = s.loc_zval[t]
        xmin, dx = -7.0, 0.0125
        n = int((np.log(10.0 * z) - xmin) / dx) + 1
        r = np.exp(xmin + dx * np.arange(n)) / z
        rc = rng.uniform(0.6, 1.0)
        a = rng.uniform(-1.5, -0.3)
        w = rng.uniform(0.6, 1.2)
        from math import erf
        v = np.array([-z * e2 * erf(ri / rc) / ri for ri in r]) + a * np.exp(-(r / w) ** 2)
        s.loc_r.append(r)
        s.loc_rab.append(r * dx)
        s.loc_v.append(v)


def check_box(s: System):
    """Every rotated (and umklapp-shifted) sphere must fit the FFT box without
    aliasing: |component| < N/2 on every axis."""
    Ainv = np.linalg.inv(s.alat)
    half = np.array(s.fft_dims) // 2
    for R in s.sym_R:
        W = s.alat.T @ R @ Ainv.T       # crystal action on reciprocal coordinates
        Wi = np.rint(W)
        if np.abs(W - Wi).max() > 1e-6:
            raise RuntimeError("symmetry is not integral on the reciprocal lattice")
        for n in s.miller:
            r = np.abs(n @ Wi.T).max(axis=0) + 1
            if np.any(r >= half):
                raise RuntimeError("FFT box too small for the plane-wave sphere")


# --------------------------------------------------------------------------
# binary container shared with the compiled reference harness
# --------------------------------------------------------------------------

_DT = {np.dtype(np.float64): 0, np.dtype(np.int32): 1, np.dtype(np.complex128): 2}


def _rec(f, name, arr):
    arr = np.ascontiguousarray(arr)
    if arr.dtype == np.int64 or arr.dtype == bool:
        arr = arr.astype(np.int32)
    code = _DT[arr.dtype]
    nb = name.encode()
    f.write(struct.pack("<32siI", nb + b"\0" * (32 - len(nb)), code, arr.ndim))
    f.write(struct.pack("<" + "q" * arr.ndim, *arr.shape))
    f.write(arr.tobytes())


def write_system(s: System, path: str, kminusq: bool = False, non_loc: bool = True):
    """Write the system as named records: 32-byte name, int32 dtype code
    (0 f64, 1 i32, 2 c128), uint32 ndim, int64 dims, raw little-endian data."""
    with open(path, "wb") as f:
        f.write(b"LELPHSYS")
        hdr = np.array([s.natom, s.ntype, len(s.sym_R), s.timerev, s.nspin, s.nspinor, s.nbnds, s.nmag,
                        s.nmodes, s.nk_ibz, s.nk_bz, *s.fft_dims, s.nltimesj, s.lmax,
                        int(s.is_soc_present), len(s.qpts), int(kminusq), int(non_loc), ord(s.dimension)],
                       np.int32)
        _rec(f, "header", hdr)
        _rec(f, "alat", s.alat)
        _rec(f, "blat", s.blat)
        _rec(f, "atom_pos", s.atom_pos)
        _rec(f, "atom_type", s.atom_type)
        _rec(f, "sym_R", s.sym_R)
        _rec(f, "sym_tau", s.sym_tau)
        _rec(f, "sym_trev", s.sym_trev.astype(np.int32))
        _rec(f, "kibz", s.kibz)
        _rec(f, "kbz_crys", s.kbz_crys)
        _rec(f, "kmap", s.kmap)
        _rec(f, "PP_table", s.PP_table)
        _rec(f, "Fsign", s.Fsign)
        _rec(f, "qpts", s.qpts)
        _rec(f, "eigVec", s.eigVec)
        _rec(f, "dVscf", s.dVscf)
        for ik in range(s.nk_ibz):
            _rec(f, f"gvec{ik}", s.gvec[ik])
            _rec(f, f"wfc{ik}", s.wfc[ik])
            _rec(f, f"Fk{ik}", s.Fk[ik])
        if s.fCoeff is not None:
            for i, fc in enumerate(s.fCoeff):
                if fc is not None:
                    _rec(f, f"fCoeff{i}", fc)
        if s.loc_zval is not None:
            _rec(f, "loc_zval", np.asarray(s.loc_zval, np.float64))
            for t in range(s.ntype):
                _rec(f, f"loc_r{t}", s.loc_r[t])
                _rec(f, f"loc_rab{t}", s.loc_rab[t])
                _rec(f, f"loc_v{t}", s.loc_v[t])
        f.write(b"END\0" + b"\0" * 28)


def read_g(path: str, s: System, nq: int) -> np.ndarray:
    raw = np.fromfile(path, dtype=np.complex128)
    return raw.reshape(nq, s.nk_bz, s.nmodes, s.nspin, s.nbnds, s.nbnds)
