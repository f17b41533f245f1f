"""GPU parity of rotate_dvscf (src/symmetries/rotate_dvscf.c:22-368) through
the C ABI: every case of tests/golden/rotate_dvscf.npz against the oracle on
the whole box (FP64, 1e-12 relative: the output is a permutation of the input
times a phase, so any index error would show as an O(1) difference) and
against the reference's samples; an operation that does not map the FFT grid
onto itself returns LELPH_GPU_ERR_GEOMETRY."""
import json
import os

import numpy as np
import pytest

import elph_oracle as O
from golden_util import GOLDEN_DIR
from letzelphc_gb300 import synth
from letzelphc_gb300.elph import LelphError, LelphGPU

pytestmark = pytest.mark.gpu


def _fixture():
    z = np.load(os.path.join(GOLDEN_DIR, "rotate_dvscf.npz"))
    return z, json.loads(str(z["cases"])), json.loads(str(z["systems"]))


def _system(systems, name):
    base, ov = systems[name]
    ov = {k: (tuple(v) if isinstance(v, list) and k in ("kgrid", "fft", "ls") else v) for k, v in ov.items()}
    return synth.make_system(base, ov)


@pytest.mark.parametrize("sysname", ["c0", "soc"])
def test_rotate_dvscf_matches_oracle_and_reference(sysname):
    z, cases, systems = _fixture()
    s = _system(systems, sysname)
    with LelphGPU(s, "fp64") as ctx:
        for name, isym, trev_ov, comp in cases:
            if name != sysname:
                continue
            trev = int(s.sym_trev[isym]) if trev_ov is None else trev_ov
            R, tau = s.sym_R[isym], s.sym_tau[isym]
            out = ctx.rotate_dvscf(s.qpts[0], R, tau, trev, comp, s.dVscf[0])
            ref = O.rotate_dvscf(s, s.qpts[0], s.dVscf[0], R, tau, trev, comp)
            assert np.abs(out - ref).max() < 1e-12 * np.abs(ref).max(), (isym, trev, comp)
            key = f"{sysname}_{isym}_{trev}_{comp}"
            smp = z[key + "_sample"]
            assert np.abs(out.reshape(-1)[::97] - smp).max() < 1e-12 * np.abs(smp).max(), key


def test_rotate_dvscf_rejects_incompatible_operation():
    z, cases, systems = _fixture()
    s = _system(systems, "c0")
    c, sn = np.cos(np.pi / 6), np.sin(np.pi / 6)
    R = np.array([[c, -sn, 0.0], [sn, c, 0.0], [0.0, 0.0, 1.0]])  # 30 degrees: not a symmetry of the grid
    with LelphGPU(s, "fp64") as ctx:
        with pytest.raises(LelphError) as e:
            ctx.rotate_dvscf(s.qpts[0], R, np.zeros(3), 0, 0, s.dVscf[0])
        assert e.value.status == -5
