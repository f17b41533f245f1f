"""CPU restatement of LetzElPhC's per-q electron-phonon matrix-element path.

TEST INFRASTRUCTURE ONLY.  This module is the checker that the CUDA path is
compared against (tests/, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py``).  Nothing in the product imports it.

It restates, in numpy FP64, the reference's G-space algorithm for one q-point
(``compute_and_write_elphq``, src/elph/compute_elph_matq.c:20-234):

* ``elph_local``        src/dvloc/compute_Vbare_loc.c:17-353
* ``add_elph_nonlocal`` src/nonloc/Vbare_nloc.c:35-577 (+ sum_VNL_KKp.c:8-58)
* ``elph_q_rotate``     src/symmetries/elphq_expand.c:16-73
* ``electronic_reps``, ``dmats`` (the Dmats that elph_driver computes before
  the q loop): src/symmetries/elec_reps.c:16-413, src/elph/compute_dmats.c:20-131
* ``compute_elphq_star`` (the q-star loop of the stage):
  src/elph/compute_elph_matq.c:116-217
* ``read_dvscf_qe`` (the dV_scf ingest after the file read):
  src/io/qe/read_dvscf.c:15-172
* ``vloc_table``, ``dvlocq``, ``add_dvscf_qe`` (the per-q local bare
  potential that elph_driver adds before the stage,
  src/elph/elph_driver.c:234-252): src/dvloc/vlocg_table.c:16-154,
  src/dvloc/VlocG_atom.c:10-57, src/common/spline.c:13-139,
  src/dvloc/dVbare_loc.c:16-231, src/dvloc/add_dvscf.c:12-92

FFTW is replaced by numpy's pocketfft: the reference's FFT is a pruned,
slab-distributed 3-D complex DFT (src/fft/*.c); pruning changes nothing but
rounding, so the full 3-D transform is used here.  Constants follow
src/common/constants.h (truncated pi = 3.1415927).

Parity of this restatement is pinned against the reference itself: the
reference's own hot-path C sources are compiled unmodified against small
single-rank MPI / FFTW / CBLAS / netCDF shims (oracle/Makefile) and the two
are compared on the golden systems of tests/golden/ (tests/test_oracle_vs_ref.py).
"""
from __future__ import annotations

import math

import numpy as np

ELPH_PI = 3.1415927
ELPH_EPS = 1e-5
ELPH_EPS6 = 1e-6
ELPH_E2 = 2.0


# ---------------------------------------------------------------- 3x3 helpers

def mat_vec3(M, v, trans=False):
    """MatVec3f, src/common/numerical_func.c:226-241 (explicit left-to-right sums)."""
    M = np.asarray(M, float).reshape(9)
    if trans:
        return np.array([M[0] * v[0] + M[3] * v[1] + M[6] * v[2],
                         M[1] * v[0] + M[4] * v[1] + M[7] * v[2],
                         M[2] * v[0] + M[5] * v[1] + M[8] * v[2]])
    return np.array([M[0] * v[0] + M[1] * v[1] + M[2] * v[2],
                     M[3] * v[0] + M[4] * v[1] + M[5] * v[2],
                     M[6] * v[0] + M[7] * v[1] + M[8] * v[2]])


def det3x3(m):
    m = np.asarray(m, float).reshape(9)
    return (m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6])
            + m[2] * (m[7] * m[3] - m[4] * m[6]))


def find_kidx_in_list(klist, kpt):
    """src/common/numerical_func.c:471-497."""
    d = klist - kpt[None, :]
    d = d - np.rint(d)
    s = np.sqrt((d * d).sum(axis=1))
    hit = np.nonzero(s < ELPH_EPS)[0]
    return int(hit[0]) if len(hit) else -1


def get_kplusq_idxs(kpts_crys, q):
    """src/common/numerical_func.c:500-524."""
    out = np.empty(len(kpts_crys), np.int64)
    for i, k in enumerate(kpts_crys):
        out[i] = find_kidx_in_list(kpts_crys, k + q)
        if out[i] < 0:
            raise ValueError("K+Q point cannot be found in kgrid")
    return out


# ------------------------------------------------------------ wfc symmetry ops

def rotate_gvecs(G, S, alat, G0=None):
    """rotateGvecs(inverse=False, crystal=True), src/wfc/rotate_Gvecs.c:15-81:
    G_crys = (alat^T S) G, plus the crystal coordinates of G0."""
    sym_temp = alat.T @ S
    out = G @ sym_temp.T
    if G0 is not None:
        out = out + mat_vec3(alat, G0, True)[None, :]
    return out


def sort_pw(gfloat, sets):
    """Sort_pw + Sorted_gvecs_idxs, src/wfc/sortpw.c:95-315, src/wfc/gsort.c:16-128:
    rint the crystal coordinates and order by x, then y, then z."""
    gi = np.rint(gfloat).astype(np.int64)
    order = np.lexsort((gi[:, 2], gi[:, 1], gi[:, 0]))
    return gi[order], sets[..., order]


def su2mat(sym, nspinor, invert, time_rev):
    """SU2mat, src/wfc/su2mat.c:16-117 (Euler angles, -i sigma_y for time reversal)."""
    if nspinor == 1:
        return np.array([1.0 + 0j, 0, 0, 1])
    det = det3x3(sym)
    s = np.asarray(sym, float).reshape(9) / det
    if abs(s[6] + 1) < ELPH_EPS:
        alpha, beta, delta = 0.0, ELPH_PI / 2.0, math.atan2(s[1], s[2])
    elif abs(s[6] - 1) < ELPH_EPS:
        alpha, beta, delta = 0.0, -ELPH_PI / 2.0, math.atan2(-s[1], -s[2])
    else:
        beta = -math.asin(s[6])
        alpha = math.atan2(s[3] / math.cos(beta), s[0] / math.cos(beta))
        delta = math.atan2(s[7] / math.cos(beta), s[8] / math.cos(beta))
    alpha, beta, delta = alpha / 2, beta / 2, delta / 2
    p0 = np.array([1, 0, 0, 1], complex)
    px = np.array([0, 1, 1, 0], complex)
    py = np.array([0, -1j, 1j, 0], complex)
    pz = np.array([1, 0, 0, -1], complex)
    sd = math.cos(delta) * p0 - 1j * math.sin(delta) * px
    sb = math.cos(beta) * p0 - 1j * math.sin(beta) * py
    sa = math.cos(alpha) * p0 - 1j * math.sin(alpha) * pz

    def mm(a, b):
        return np.array([a[0] * b[0] + a[1] * b[2], a[0] * b[1] + a[1] * b[3],
                         a[2] * b[0] + a[3] * b[2], a[2] * b[1] + a[3] * b[3]])
    u = mm(sa, mm(sb, sd))
    if time_rev:
        a1, b1, c1, d1 = u
        u = np.array([-c1, -d1, a1, b1])
    if invert:
        u = np.array([np.conj(u[0]), np.conj(u[2]), np.conj(u[1]), np.conj(u[3])])
    return u


def su2rotate(su2, wfc):
    """src/wfc/su2rotate.c:13-41; wfc (..., nspinor, npw)."""
    if wfc.shape[-2] != 2:
        return wfc
    up = wfc[..., 0, :]
    dw = wfc[..., 1, :]
    out = np.empty_like(wfc)
    out[..., 0, :] = up * su2[0] + dw * su2[1]
    out[..., 1, :] = up * su2[2] + dw * su2[3]
    return out


def apply_trans_wfc(tau, kvec, gvecs, wfc, conjugate=False):
    """src/wfc/trans_wfc.c:15-52: c(G) e^{-i 2pi k.tau} e^{-i 2pi G.tau}."""
    kphase = np.exp(-1j * 2 * ELPH_PI * float(kvec[0] * tau[0] + kvec[1] * tau[1] + kvec[2] * tau[2]))
    gdot = gvecs[:, 0] * tau[0] + gvecs[:, 1] * tau[1] + gvecs[:, 2] * tau[2]
    ph = kphase * np.exp(-1j * 2 * ELPH_PI * gdot)
    out = wfc * ph
    return np.conj(out) if conjugate else out


# ------------------------------------------------------------------ FFTs

def box_index(gint, fft_dims):
    Nx, Ny, Nz = fft_dims
    return ((gint[:, 0] % Nx) * Ny + (gint[:, 1] % Ny)) * Nz + (gint[:, 2] % Nz)


def invfft3d(gint, wfcG, fft_dims, conjugate):
    """invfft3D, src/fft/bwdfft.c:13-120: sphere -> box (conj if asked), then
    the unnormalised backward DFT.  wfcG (nsets, npw) -> (nsets, Nx, Ny, Nz)."""
    Nx, Ny, Nz = fft_dims
    N = Nx * Ny * Nz
    box = np.zeros((wfcG.shape[0], N), complex)
    box[:, box_index(gint, fft_dims)] = np.conj(wfcG) if conjugate else wfcG
    box = box.reshape(-1, Nx, Ny, Nz)
    return np.fft.ifftn(box, axes=(1, 2, 3)) * N


def fft_convolution3d(gint, nspinor, nmag, Vr, psir, fft_dims):
    """fft_convolution3D, src/fft/convolution.c:13-189: FFT[dV psi] * 1/N on the
    sphere.  Vr (nmag_avail, Nx, Ny, Nz), psir (nbnd, nspinor, Nx, Ny, Nz)
    -> (nbnd, nspinor, npw)."""
    if nspinor == 1:
        nmag = 1
    Nx, Ny, Nz = fft_dims
    N = Nx * Ny * Nz
    idx = box_index(gint, fft_dims)
    out = np.empty((psir.shape[0], nspinor, len(gint)), complex)
    for isp in range(nspinor):
        if nmag == 1:
            prod = psir[:, isp] * Vr[0][None]
        else:
            d0 = Vr[2 * isp]
            d1 = Vr[2 * isp + 1]
            prod = psir[:, 0] * d0[None] + psir[:, 1] * d1[None]
        f = np.fft.fftn(prod, axes=(1, 2, 3)).reshape(prod.shape[0], N)
        out[:, isp] = f[:, idx] * (1.0 / N)
    return out


# -------------------------------------------------------------- local part

def elph_local(qpt, s, ikq, ik, kqsym, ksym, dVlocr):
    """elphLocal, src/dvloc/compute_Vbare_loc.c:17-353.
    dVlocr (nmodes, nmag, Nx, Ny, Nz) -> g (nmodes, nspin, nb_k, nb_kq)."""
    nspin, nb, nspinor, nmag = s.nspin, s.nbnds, s.nspinor, s.nmag
    lat = s.alat
    blat = s.blat
    wfc_kq, Gkq = s.wfc[ikq], s.gvec[ikq]
    wfc_k, Gk = s.wfc[ik], s.gvec[ik]
    kqvec, kvec = s.kibz[ikq], s.kibz[ik]
    symkq, symk = s.sym_R[kqsym], s.sym_R[ksym]
    taukq, tauk = s.sym_tau[kqsym], s.sym_tau[ksym]
    trkq, trk = bool(s.sym_trev[kqsym]), bool(s.sym_trev[ksym])

    tempSkq = mat_vec3(symkq, kqvec)                       # :103
    tempSk = mat_vec3(symk, kvec)                          # :104
    kvecSk = mat_vec3(lat, tempSk, True)                   # :106
    kvecSkq = kvecSk + np.asarray(qpt, float)              # :108-111
    tempSkq = tempSkq - tempSk                             # :114-117
    qcart = mat_vec3(blat, qpt) / (2 * ELPH_PI)            # :120-125
    taukq_crys = mat_vec3(blat, taukq, True) / (2 * ELPH_PI)
    tauk_crys = mat_vec3(blat, tauk, True) / (2 * ELPH_PI)
    ulm = tempSkq - qcart                                  # :141-144

    gSkq = rotate_gvecs(Gkq, symkq, lat, ulm)              # :146
    gSk = rotate_gvecs(Gk, symk, lat, None)                # :147
    su2kq = su2mat(symkq, nspinor, False, trkq)
    su2k = su2mat(symk, nspinor, False, trk)

    gkq_i, wkq = sort_pw(gSkq, wfc_kq)                     # :170-176
    gk_i, wk = sort_pw(gSk, wfc_k)

    # k+q: su2 + fractional translation (:197-205)
    wkq = su2rotate(su2kq, wkq)
    wkq = apply_trans_wfc(taukq_crys, kvecSkq, gkq_i.astype(float), wkq)
    # k: su2 + translation + (conj) inverse FFT (:223-241)
    wk = su2rotate(su2k, wk)
    wk = apply_trans_wfc(tauk_crys, kvecSk, gk_i.astype(float), wk)
    Nx, Ny, Nz = s.fft_dims
    psir = invfft3d(gk_i, wk.reshape(-1, len(gk_i)), s.fft_dims, trk)
    psir = psir.reshape(nspin, nb, nspinor, Nx, Ny, Nz)

    if nmag == 2 and (nspin != 2 or nspinor != 1):
        raise ValueError("Incompatible dvscf")
    out = np.zeros((s.nmodes, nspin, nb, nb), complex)
    for iv in range(s.nmodes):
        for isp in range(nspin):
            Vr = dVlocr[iv, isp:] if nmag == 2 else dVlocr[iv]
            dvpsi = fft_convolution3d(gkq_i, nspinor, nmag, Vr, psir[isp], s.fft_dims)
            A = dvpsi.reshape(nb, -1)
            B = wkq[isp].reshape(nb, -1)
            out[iv, isp] = A @ (B.T if trkq else np.conj(B).T)   # 'T' / 'C' (:312-326)
    return out


# ----------------------------------------------------------- nonlocal part

def _factorial(n):
    return math.gamma(n + 1)


def legendre(l, m, x):
    """Associated Legendre without Condon-Shortley, src/common/numerical_func.c:29-94."""
    if l == 0 and m == 0:
        return 1.0
    if l < 0:
        return legendre(-l - 1, m, x)
    if abs(m) > l:
        return 0.0
    if m < 0:
        return legendre(l, -m, x) * (-1.0) ** (-m) * _factorial(l + m) / _factorial(l - m)
    val = 1.0
    sq = math.sqrt(1 - x * x)
    for im in range(1, m + 1):
        val *= (2 * im - 1) * sq
    if l == m:
        return val
    vmm = val
    val *= (2 * m + 1) * x
    if l == m + 1:
        return val
    for im in range(m + 2, l + 1):
        tmp = val
        val = (2 * im - 1) * x * val - (im + m - 1) * vmm
        val = val / (im - m)
        vmm = tmp
    return val


def ylm(l, m, v):
    """Real spherical harmonics (Blanco et al.), src/common/numerical_func.c:97-152."""
    if l < 0:
        return 0.0
    norm = math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    if norm < ELPH_EPS6:
        return 0.0 if l != 0 else 1.0 / math.sqrt(4 * ELPH_PI)
    cost = v[2] / norm
    phi = math.atan2(v[1], v[0])
    if m > 0:
        sh = math.sqrt(2) * math.cos(m * phi)
    elif m < 0:
        m = -m
        sh = math.sqrt(2) * math.sin(m * phi)
    else:
        sh = 1.0
    sh *= legendre(l, m, cost)
    sh *= math.sqrt(_factorial(l - m) * (2 * l + 1) / (4 * ELPH_PI * _factorial(l + m)))
    return sh


def ylm_vec(l, m, V):
    return np.array([ylm(l, m, v) for v in V])


def sum_vnl_kkp(K, Kp, f, nspin, nb, nspinor, out):
    """sum_VNL_KKp, src/nonloc/sum_VNL_KKp.c:8-58.
    K, Kp (4, nspin, nb, nspinor); out (3, nspin, nb_k, nb_kq)."""
    for ix in range(3):
        for s1 in range(nspinor):
            for s2 in range(nspinor):
                fc = f[nspinor * s1 + s2]
                # out[ix, is, ib1 (k), ib2 (kq)] += f (K[ix+1][ib2,s1] Kp[0][ib1,s2] + K[0][ib2,s1] Kp[ix+1][ib1,s2])
                out[ix] += fc * (Kp[0, :, :, s2][:, :, None] * K[ix + 1, :, :, s1][:, None, :]
                                 + Kp[ix + 1, :, :, s2][:, :, None] * K[0, :, :, s1][:, None, :])


def add_elph_nonlocal(s, ikq, ik, kqsym, ksym, eigVec, elph):
    """add_elphNonLocal, src/nonloc/Vbare_nloc.c:35-577.  Adds into elph
    (nmodes, nspin, nb_k, nb_kq)."""
    nspin, nb, nspinor = s.nspin, s.nbnds, s.nspinor
    ntype, natom = s.ntype, s.natom
    lmax = s.lmax
    PP = s.PP_table
    wK = s.wfc[ikq].copy()
    wKp = s.wfc[ik].copy()
    SK, SKp = s.sym_R[kqsym], s.sym_R[ksym]
    tauK, tauKp = s.sym_tau[kqsym], s.sym_tau[ksym]
    trK, trKp = bool(s.sym_trev[kqsym]), bool(s.sym_trev[ksym])
    # rotate k+G (:148-168)
    GK = (s.gvec[ikq] + s.kibz[ikq][None, :]) @ SK.T
    GKp = (s.gvec[ik] + s.kibz[ik][None, :]) @ SKp.T
    YK = {(l, m): ylm_vec(l, m, GK) for l in range(lmax + 1) for m in range(-l, l + 1)}
    YKp = {(l, m): ylm_vec(l, m, GKp) for l in range(lmax + 1) for m in range(-l, l + 1)}
    su2K = su2mat(SK, nspinor, False, trK)
    su2Kp = su2mat(SKp, nspinor, False, trKp)
    zero = np.zeros(3)
    wK = apply_trans_wfc(tauK, zero, GK, su2rotate(su2K, wK))       # :227-235
    wKp = apply_trans_wfc(tauKp, zero, GKp, su2rotate(su2Kp, wKp))  # :237-245
    FK, FKp = s.Fk[ikq], s.Fk[ik]
    nsets = nspin * nb * nspinor
    BK = wK.reshape(nsets, -1)
    BKp = wKp.reshape(nsets, -1)
    buf = np.zeros((natom, 3, nspin, nb, nb), complex)
    for ia in range(natom):
        it = s.atom_type[ia]
        tau = s.atom_pos[ia]
        betaK, betaKp, channels = [], [], []
        for lidx in range(s.nltimesj):
            l = int(np.rint(PP[lidx, it, 0] - 1))
            if l < 0:
                continue
            sign = s.Fsign[lidx, it]
            dotK = GK[:, 0] * tau[0] + GK[:, 1] * tau[1] + GK[:, 2] * tau[2]
            dotKp = GKp[:, 0] * tau[0] + GKp[:, 1] * tau[1] + GKp[:, 2] * tau[2]
            for im in range(2 * l + 1):
                b0 = FK[lidx, it] * np.exp(-1j * 2 * ELPH_PI * dotK) * YK[(l, im - l)]
                betaK.append(np.stack([b0, b0 * GK[:, 0] * sign, b0 * GK[:, 1] * sign, b0 * GK[:, 2] * sign]))
            for im in range(2 * l + 1):
                b0 = FKp[lidx, it] * np.exp(1j * 2 * ELPH_PI * dotKp) * YKp[(l, im - l)]
                betaKp.append(np.stack([b0, -b0 * GKp[:, 0] * sign, -b0 * GKp[:, 1] * sign, -b0 * GKp[:, 2] * sign]))
            channels.append((lidx, l))
        betaK = np.array(betaK)      # (nproj, 4, npwK)
        betaKp = np.array(betaKp)
        bandK = betaK @ (BK.T if trK else np.conj(BK).T)       # :412-414 ('C' or 'T')
        bandKp = betaKp @ (np.conj(BKp).T if trKp else BKp.T)  # :416-418 ('T' or 'C')
        bandK = bandK.reshape(-1, 4, nspin, nb, nspinor)
        bandKp = bandKp.reshape(-1, 4, nspin, nb, nspinor)
        ilc = 0
        for (lidx, l) in channels:
            j = int(np.rint(PP[lidx, it, 1]))
            soc_fac = 1.0
            if j != 0 and not s.is_soc_present:
                soc_fac = (j + 1.0) / (4.0 * l + 2.0)
            fc = None
            if s.fCoeff is not None:
                fc = s.fCoeff[s.ntype * lidx + it]
            for im1 in range(2 * l + 1):
                for im2 in range(2 * l + 1):
                    if fc is None and im1 != im2:
                        continue
                    if fc is None:
                        f = np.array([soc_fac, 0, 0, soc_fac], complex)
                    else:
                        f = fc[im1, im2].reshape(-1)
                    sum_vnl_kkp(bandK[ilc + im1], bandKp[ilc + im2], f, nspin, nb, nspinor, buf[ia])
            ilc += 2 * l + 1
    pre = -2 * ELPH_PI * 1j * ELPH_E2
    elph += pre * np.einsum("vj,jsmn->vsmn", eigVec.reshape(s.nmodes, natom * 3),
                            buf.reshape(natom * 3, nspin, nb, nb))
    return elph


# -------------------------------------------------------------- q stage

def compute_elphq(s, iq, eigVec=None, dVscfq=None, non_loc=True, kminusq=False, k_list=None):
    """compute_and_write_elphq for one iBZ q, src/elph/compute_elph_matq.c:20-234.
    Returns g (nk, nmodes, nspin, nb, nb) for the full-BZ k indices of
    ``k_list`` (all of them by default)."""
    qpt = np.asarray(s.qpts[iq], float)
    eigVec = s.eigVec[iq] if eigVec is None else eigVec
    dVscfq = s.dVscf[iq] if dVscfq is None else dVscfq
    qt = -qpt if kminusq else qpt
    kpq = get_kplusq_idxs(s.kbz_crys, qt)
    ks = range(s.nk_bz) if k_list is None else k_list
    out = np.zeros((len(ks), s.nmodes, s.nspin, s.nbnds, s.nbnds), complex)
    for ii, i in enumerate(ks):
        idx_k, idx_kq = i, int(kpq[i])
        if kminusq:
            idx_k, idx_kq = idx_kq, idx_k
        ik, ksym = s.kmap[idx_k]
        ikq, kqsym = s.kmap[idx_kq]
        g = elph_local(qpt, s, ikq, ik, kqsym, ksym, dVscfq)
        if non_loc:
            add_elph_nonlocal(s, ikq, ik, kqsym, ksym, eigVec, g)
        out[ii] = g
    return out


def elph_q_rotate(Dl, g, Dr, tim_rev):
    """elph_q_rotate, src/symmetries/elphq_expand.c:16-73.
    g (nmodes, nspin, nb, nb); D (nspin, nb, nb)."""
    out = np.empty_like(g)
    for isp in range(g.shape[1]):
        for iv in range(g.shape[0]):
            gq = g[iv, isp]
            A = np.conj(gq).T if tim_rev else gq.T
            tmp = A @ np.conj(Dr[isp]).T
            out[iv, isp] = tmp.T @ Dl[isp].T
    return out


# ---------------------------------------------- electronic representations

def kbz_cart(s):
    """Cartesian full-BZ k-points as the lattice struct holds them:
    blat k_crys / (2 pi) with the reference's pi."""
    return s.kbz_crys @ s.blat.T / (2 * ELPH_PI)


def electronic_reps(s, R, tauR, trevR, ikBZ):
    """electronic_reps, src/symmetries/elec_reps.c:16-413:
    D[spin, b, a] = <psi_{Rk, b} | U(R) | psi_{k, a}>, with Rk = S2 k2 and
    k = S1 k1 unfolded from the irreducible wedge (kmap), the S2 k2
    coefficients reordered onto the R S1 k1 plane-wave list (find_gvecs_idxs,
    src/wfc/gsort.c:49-93; unmatched entries zero) and
    D = (conj-prepared S2 k2 rows) @ (R S1 k1 rows)^T (elec_reps.c:375-392)."""
    alat, blat = s.alat, s.blat
    R = np.asarray(R, float)
    kcart = kbz_cart(s)
    Rk = mat_vec3(alat, mat_vec3(R, kcart[ikBZ]), True)                      # :35-38
    iRk = find_kidx_in_list(s.kbz_crys, Rk)                                   # :41-49
    if iRk < 0:
        raise ValueError("Rotated k point not found")
    ik1, isym1 = (int(v) for v in s.kmap[ikBZ])                               # :66-70
    ik2, isym2 = (int(v) for v in s.kmap[iRk])
    S1, tau1, tr1 = s.sym_R[isym1], s.sym_tau[isym1], bool(s.sym_trev[isym1])
    S2, tau2, tr2 = s.sym_R[isym2], s.sym_tau[isym2], bool(s.sym_trev[isym2])
    k1, k2 = s.kibz[ik1], s.kibz[ik2]
    kcrys = mat_vec3(alat, mat_vec3(S1, k1), True)                            # :94-97
    tcr = [mat_vec3(blat, t, True) / (2 * ELPH_PI) for t in (tau1, tauR, tau2)]  # :100-109
    su1 = su2mat(S1, s.nspinor, False, tr1)                                   # :128-134
    suR = su2mat(R, s.nspinor, False, trevR)
    su2_ = su2mat(S2, s.nspinor, False, tr2)
    RS1 = R @ S1                                                              # :146
    RS1k1 = mat_vec3(RS1, k1)
    ulm = mat_vec3(S2, k2) - RS1k1                                            # :149-161
    Rkcrys = mat_vec3(alat, RS1k1, True)
    G_S1k1 = rotate_gvecs(s.gvec[ik1], S1, alat)                              # :165-171
    G_RS1k1 = rotate_gvecs(s.gvec[ik1], RS1, alat)
    G_S2k2 = rotate_gvecs(s.gvec[ik2], S2, alat, ulm)
    pos = {tuple(v): i for i, v in enumerate(np.rint(G_RS1k1).astype(np.int64))}
    idx = np.array([pos.get(tuple(v), -1) for v in np.rint(G_S2k2).astype(np.int64)])
    nsp, nb, ns = s.nspin, s.nbnds, s.nspinor
    w1 = s.wfc[ik1].reshape(nsp * nb, ns, -1)
    w2 = s.wfc[ik2].reshape(nsp * nb, ns, -1)
    a = su2rotate(su1, w1)                                                    # :311-316
    a = apply_trans_wfc(tcr[0], kcrys, G_S1k1, a, tr1)
    a = su2rotate(suR, a)                                                     # :321-325
    a = apply_trans_wfc(tcr[1], Rkcrys, G_RS1k1, a, trevR)
    b = np.zeros_like(w1)                                                     # :331-361
    hit = idx >= 0
    b[:, :, idx[hit]] = w2[:, :, hit]
    b = su2rotate(su2_, b)                                                    # :364-372
    b = apply_trans_wfc(tcr[2], Rkcrys, G_RS1k1, b, not tr2)
    a = a.reshape(nsp, nb, -1)
    b = b.reshape(nsp, nb, -1)
    return np.einsum("sbk,sak->sba", b, a)                                    # :375-392


def dmats(s, sym_R=None, sym_tau=None, sym_trev=None, pairs=None):
    """compute_and_write_dmats, src/elph/compute_dmats.c:20-131: D for every
    (symmetry, full-BZ k) in (isym, ik) order, (nsym, nk, nspin, nb, nb); with
    ``pairs`` only those (isym, ik)."""
    sym_R = s.sym_R if sym_R is None else sym_R
    sym_tau = s.sym_tau if sym_tau is None else sym_tau
    sym_trev = s.sym_trev if sym_trev is None else sym_trev
    if pairs is None:
        pairs = [(i, k) for i in range(len(sym_R)) for k in range(len(s.kbz_crys))]
    return np.array([electronic_reps(s, sym_R[i], sym_tau[i], bool(sym_trev[i]), k) for i, k in pairs])


def q_star(s, qpt, sym_R=None):
    """Members of the star of q (crystal) under the phonon symmetries, each
    with the first symmetry that produces it, identity first: the (qmap,
    nqstar) a phonon code hands to the stage for this q."""
    sym_R = s.sym_R if sym_R is None else sym_R
    qc = np.linalg.solve(s.alat.T, np.asarray(qpt, float))  # crystal -> cartesian (no 2 pi)
    members, syms = [], []
    for i, R in enumerate(sym_R):
        sq = mat_vec3(s.alat, mat_vec3(R, qc), True)
        if find_kidx_in_list(np.array(members).reshape(-1, 3), sq) < 0:
            members.append(sq)
            syms.append(i)
    return np.array(members), np.array(syms, np.int32)


def compute_elphq_star(s, iq, star_syms, D, eigVec=None, dVscfq=None, non_loc=True, kminusq=False):
    """compute_and_write_elphq with its q-star loop, src/elph/compute_elph_matq.c:116-217:
    row 0 is g(q, k) at k; row istar holds
    elph_q_rotate(D[S][k+q], g(q, k), D[S][k], time_rev(S)) at S k, S = star_syms[istar].
    D: Dmats (nsym, nk, nspin, nb, nb).  Returns (nstar, nk, nmodes, nspin, nb, nb)."""
    qpt = np.asarray(s.qpts[iq], float)
    g = compute_elphq(s, iq, eigVec, dVscfq, non_loc, kminusq)
    qt = -qpt if kminusq else qpt
    kpq = get_kplusq_idxs(s.kbz_crys, qt)
    kcart = kbz_cart(s)
    out = np.zeros((len(star_syms),) + g.shape, complex)
    out[0] = g
    for i in range(s.nk_bz):
        idx_k, idx_kq = i, int(kpq[i])
        if kminusq:
            idx_k, idx_kq = idx_kq, idx_k
        for istar in range(1, len(star_syms)):
            S = int(star_syms[istar])
            gs = elph_q_rotate(D[S, idx_kq], g[i], D[S, idx_k], bool(s.sym_trev[S]))
            sk = mat_vec3(s.alat, mat_vec3(s.sym_R[S], kcart[i]), True)
            isk = find_kidx_in_list(s.kbz_crys, sk)
            if isk < 0:
                raise ValueError("Unable to to find S*k index")
            out[istar, isk] = gs
    return out


def read_dvscf_qe(raw, eig, pats, nmag, fft_dims):
    """read_dvscf_qe after the file read, src/io/qe/read_dvscf.c:15-172: raw
    (patterns, nmag, Nz, Ny, Nx) -> (x, y, z), then the mode basis
    dV_nu = sum_p (eig pats^H)[nu][p] dV_p.  Returns (nmodes, nmag, Nx, Ny, Nz)."""
    Nx, Ny, Nz = fft_dims
    nm = eig.shape[0]
    d = np.asarray(raw).reshape(nm, nmag, Nz, Ny, Nx).transpose(0, 1, 4, 3, 2)
    M = eig.reshape(nm, -1) @ np.conj(np.asarray(pats).reshape(nm, -1)).T
    return np.einsum("vp,pmxyz->vmxyz", M, d)


# ------------------------------------------------------- local bare potential

def simpson_weights(n):
    """Weights w with  sum_i w_i f_i dx_i / 3  = the reference's Simpson rule
    (src/common/numerical_func.c:155-192), including its even-n end correction."""
    w = np.zeros(n)
    if n < 3:
        return w
    w[0] = 1.0
    w[1:n - 1:2] += 4.0
    w[2:n - 1:2] += 2.0
    if n % 2:
        w[n - 1] += 1.0
    else:
        w[n - 3] -= 0.25
        w[n - 2] += 1.0
        w[n - 1] += 1.25
    return w


def vloc_gspace(G, r, rab, vloc, zval, volume, cutoff="3", eta=1.0):
    """4 pi / V int dr (sin(G r)/G) (r V_loc(r) + e2 Z erf(sqrt(eta) r)) for an
    array of |G| (src/dvloc/VlocG_atom.c:10-57); at G = 0 the sin(Gr)/G factor
    is r, and in 3-D the erf is dropped there."""
    from scipy.special import erf
    G = np.atleast_1d(np.asarray(G, float))
    w = simpson_weights(len(r)) * rab
    out = np.empty(len(G))
    base = r * vloc + ELPH_E2 * zval * erf(r * math.sqrt(eta))
    base0 = r * vloc + ELPH_E2 * zval
    for c0 in range(0, len(G), 512):
        g = G[c0:c0 + 512, None]
        small = g < ELPH_EPS
        fac = np.where(small, r[None, :], np.sin(r[None, :] * g) / np.where(small, 1.0, g))
        body = np.where(small & (cutoff == "3"), base0[None, :], base[None, :])
        out[c0:c0 + 512] = (fac * body) @ w / 3.0
    return 4 * ELPH_PI * out / volume


def prepare_spline(x, y):
    """Slopes of the not-a-knot cubic spline through (x, y)
    (src/common/spline.c:30-139: tridiagonal system, Thomas algorithm)."""
    n = len(x)
    a = np.zeros(n); b = np.zeros(n); c = np.zeros(n); d = np.zeros(n)
    dx1 = x[1] - x[0]; s1 = (y[1] - y[0]) / dx1
    dx2 = x[2] - x[1]; s2 = (y[2] - y[1]) / dx2
    a[0] = dx2 * dx2; b[0] = dx2 * dx2 - dx1 * dx1; c[0] = -dx1 * dx1
    d[0] = 2 * (s1 * dx2 * dx2 - s2 * dx1 * dx1)
    dx1 = x[n - 2] - x[n - 3]; s1 = (y[n - 2] - y[n - 3]) / dx1
    dx2 = x[n - 1] - x[n - 2]; s2 = (y[n - 1] - y[n - 2]) / dx2
    a[n - 1] = dx2 * dx2; b[n - 1] = dx2 * dx2 - dx1 * dx1; c[n - 1] = -dx1 * dx1
    d[n - 1] = 2 * (s1 * dx2 * dx2 - s2 * dx1 * dx1)
    dxi = x[2:] - x[1:-1]; dxn = x[1:-1] - x[:-2]
    si = (y[2:] - y[1:-1]) / dxi; sn = (y[1:-1] - y[:-2]) / dxn
    a[1:-1] = dxi; b[1:-1] = 2.0 * (dxi + dxn); c[1:-1] = dxn; d[1:-1] = 3 * (sn * dxi + si * dxn)
    al = -c[0] / c[1]
    a[0] += al * a[1]; b[0] += al * b[1]; c[0] += al * c[1]; d[0] += al * d[1]
    c[0] = b[0]; b[0] = a[0]; a[0] = 0.0
    al = -a[n - 1] / a[n - 2]
    a[n - 1] += al * a[n - 2]; b[n - 1] += al * b[n - 2]; c[n - 1] += al * c[n - 2]; d[n - 1] += al * d[n - 2]
    a[n - 1] = b[n - 1]; b[n - 1] = c[n - 1]; c[n - 1] = 0.0
    for i in range(1, n):
        ww = a[i] / b[i - 1]
        b[i] -= ww * c[i - 1]
        d[i] -= ww * d[i - 1]
    dy = np.zeros(n)
    dy[n - 1] = d[n - 1] / b[n - 1]
    for i in range(n - 2, -1, -1):
        dy[i] = (d[i] - c[i] * dy[i + 1]) / b[i]
    return dy


def spline_interpolate(xq, idx, x, y, dy):
    """Cubic Hermite form of the spline on [x_idx, x_idx+1] (src/common/spline.c:13-28)."""
    h = x[idx + 1] - x[idx]
    t = (xq - x[idx]) / h
    ax = dy[idx] * h - (y[idx + 1] - y[idx])
    bx = -dy[idx + 1] * h + (y[idx + 1] - y[idx])
    return (1 - t) * y[idx] + t * y[idx + 1] + t * (1 - t) * ((1 - t) * ax + t * bx)


def vloc_table(s, qmax_abs):
    """|G| grid and V_loc(|G|) table with spline slopes per species
    (create_vlocg_table, src/dvloc/vlocg_table.c:16-154)."""
    volume = abs(det3x3(s.alat))
    blat = np.asarray(s.blat)
    bi = np.sqrt((blat ** 2).sum(axis=0))
    bmin, bmax = bi.min(), bi.max()
    nmax = max(s.fft_dims)
    if bmin > 0.01:
        bmin = 0.01
    gmax = (1.7 * (nmax + 4.0) + 3 * abs(qmax_abs)) * bmax
    npts = int(math.ceil(gmax / bmin))
    dg = gmax / (npts - 1.0)
    g = np.arange(npts) * dg
    vals, slopes = [], []
    for t in range(s.ntype):
        v = vloc_gspace(g, s.loc_r[t], s.loc_rab[t], s.loc_v[t], s.loc_zval[t], volume, s.dimension)
        vals.append(v)
        slopes.append(prepare_spline(g, v))
    return {"g": g, "dg": dg, "v": np.array(vals), "dv": np.array(slopes), "volume": volume}


def miller_of_index(N):
    """FFT index -> Miller index (get_miller_idx, src/common/numerical_func.c:436-448)."""
    i = np.arange(N)
    mid = (N - 1) // 2 + 1
    return np.where(i < mid, i, (i - mid) - N // 2)


def dvlocq(s, qpt, eigVec, table):
    """Local bare potential change per mode in real space, (nmodes, Nx, Ny, Nz)
    (dVlocq, src/dvloc/dVbare_loc.c:16-231)."""
    Nx, Ny, Nz = s.fft_dims
    mx, my, mz = miller_of_index(Nx), miller_of_index(Ny), miller_of_index(Nz)
    M = np.stack(np.meshgrid(mx + qpt[0], my + qpt[1], mz + qpt[2], indexing="ij"), -1).reshape(-1, 3)
    qG = M @ np.asarray(s.blat).T                      # blat . (G + q), 2 pi included
    nrm = np.sqrt((qG ** 2).sum(1))
    g = table["g"]
    if nrm.max() > g[-1]:
        raise ValueError("Vlocg interpolation out of bounds")
    idx = np.floor(nrm / table["dg"]).astype(int)
    cut = np.ones_like(nrm)
    if s.dimension == "2":
        c = s.alat[2, 2]
        gp = np.sqrt(qG[:, 0] ** 2 + qG[:, 1] ** 2)
        cs = np.cos(qG[:, 2] * c * 0.5)
        big = gp > ELPH_EPS
        cs = np.where(big, cs - np.sin(qG[:, 2] * c * 0.5) * qG[:, 2] / np.where(big, gp, 1.0), cs)
        cut = 1 - np.exp(-c * gp * 0.5) * cs
    V = np.empty((s.ntype, len(nrm)))
    for t in range(s.ntype):
        v = spline_interpolate(nrm, idx, g, table["v"][t], table["dv"][t])
        lr = (4 * ELPH_PI * ELPH_E2) * s.loc_zval[t] * np.exp(-nrm * nrm * 0.25) * cut / \
            (np.where(nrm >= ELPH_EPS, nrm * nrm, 1.0) * table["volume"])
        V[t] = np.where(nrm >= ELPH_EPS, v - lr, v)
    cart = np.empty((len(nrm), 3 * s.natom), complex)
    for a in range(s.natom):
        fac = -1j * np.exp(-1j * (qG @ s.atom_pos[a])) * V[s.atom_type[a]]
        cart[:, 3 * a:3 * a + 3] = fac[:, None] * qG
    VG = (np.asarray(eigVec) @ cart.T).reshape(-1, Nx, Ny, Nz)
    return np.fft.ifftn(VG, axes=(1, 2, 3)) * (Nx * Ny * Nz)


def add_dvscf_qe(dv, vloc, nmag):
    """dV_scf (nmodes, nmag, ...) plus the local bare part, with the nmag = 4
    composite [V + Bz, Bx - iBy, Bx + iBy, V - Bz] (src/dvloc/add_dvscf.c:12-92)."""
    out = np.array(dv, complex, copy=True)
    for m in range(2 if nmag == 2 else 1):
        out[:, m] += vloc
    if nmag == 4:
        V, Bx, By, Bz = out[:, 0].copy(), out[:, 1].copy(), out[:, 2].copy(), out[:, 3].copy()
        out[:, 0] = V + Bz
        out[:, 1] = Bx - 1j * By
        out[:, 2] = Bx + 1j * By
        out[:, 3] = V - Bz
    return out


# ------------------------------------------------------ dV rotation (star of q)

def rotate_dvscf_index(s, R, tau, trev):
    """FFT-box permutation of rotate_dvscf (src/symmetries/rotate_dvscf.c:118-205):
    point i of the output takes point rot_idx[i] of the input.  Raises if the
    operation does not map the FFT grid onto itself."""
    blat = np.asarray(s.blat, float)
    alat = np.asarray(s.alat, float)
    tau_red = blat.T @ np.asarray(tau, float) / (2 * ELPH_PI)
    tmp = np.asarray(R, float).T @ alat / (2 * ELPH_PI)
    if trev:
        tau_red = -tau_red
        tmp = -tmp
    sym_red = blat.T @ tmp
    N = np.array(s.fft_dims)
    ii = np.stack(np.meshgrid(*[np.arange(n) for n in N], indexing="ij"), -1).reshape(-1, 3).astype(float)
    t = ii / N - tau_red
    x = t @ sym_red.T
    x = x - np.floor(x)
    x = x - np.floor(x + ELPH_EPS)
    x = x - ELPH_EPS
    x = x * N
    diff = x - np.rint(x)
    if np.any(np.abs(diff) > 1e-3 + 5e-5 * np.abs(x)):
        raise ValueError("Symmetry operation is incompatible with FFT grid.")
    r = np.rint(x).astype(np.int64)
    return (r[:, 0] * N[1] + r[:, 1]) * N[2] + r[:, 2]


def rotate_dvscf(s, qpt, dv_in, R, tau, trev, composite):
    """dV_scf of S q from dV_scf of q, (nmodes, nmag, Nx, Ny, Nz)
    (rotate_dvscf, src/symmetries/rotate_dvscf.c:22-368): permutation of the
    box, phase e^{-i (S q).tau}, for nmag = 4 the spin rotation
    U (V + B.sigma) U^dagger (inputs in the [V, Bx, By, Bz] form unless
    `composite`), complex conjugate for time-reversed operations."""
    idx = rotate_dvscf_index(s, R, tau, trev)
    qc = np.asarray(s.blat, float) @ np.asarray(qpt, float)
    Rq = np.asarray(R, float) @ qc
    ph = np.exp(-1j * float(Rq @ np.asarray(tau, float)))
    nm, nmag = dv_in.shape[:2]
    flat = dv_in.reshape(nm, nmag, -1)
    out = ph * flat[:, :, idx]
    if nmag == 4:
        u = su2mat(R, s.nspinor, False, trev)
        d0, d1, d2, d3 = (out[:, i].copy() for i in range(4))
        if not composite:
            d0, d1, d2, d3 = d0 + d3, d1 - 1j * d2, d1 + 1j * d2, d0 - d3
        cu = np.conj(u)
        m0 = u[0] * (d0 * cu[0] + d1 * cu[1]) + u[1] * (d2 * cu[0] + d3 * cu[1])
        m1 = u[0] * (d0 * cu[2] + d1 * cu[3]) + u[1] * (d2 * cu[2] + d3 * cu[3])
        m2 = u[2] * (d0 * cu[0] + d1 * cu[1]) + u[3] * (d2 * cu[0] + d3 * cu[1])
        m3 = u[2] * (d0 * cu[2] + d1 * cu[3]) + u[3] * (d2 * cu[2] + d3 * cu[3])
        if composite:
            out = np.stack([m0, m1, m2, m3], 1)
        else:
            out = np.stack([(m0 + m3) / 2, (m1 + m2) / 2, -1j * (m2 - m1) / 2, (m0 - m3) / 2], 1)
    if trev:
        out = np.conj(out)
    return out.reshape(dv_in.shape)
