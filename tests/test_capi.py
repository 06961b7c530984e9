"""CPU-only checks of the C-ABI library and the host-side logic (no GPU calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle as O
from commit_gb300 import _lib
from commit_gb300.solvers import RegSpec, level_schedule

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _ensure_built():
    if not os.path.exists(_lib.LIB_PATH):
        from commit_gb300 import build
        build.build()


def test_library_exports_every_declared_symbol():
    _ensure_built()
    names = _lib.exported_symbols()
    assert len(names) >= 15
    L = ctypes.CDLL(_lib.LIB_PATH)
    for n in names:
        assert hasattr(L, n), n
    # every declaration in include/*.h is a cgb_ function that the library exports
    for h in os.listdir(os.path.join(ROOT, 'include')):
        for line in open(os.path.join(ROOT, 'include', h)):
            m = re.match(r'^\s*(?:int|const char \*)\s*(cgb_\w+)\s*\(', line)
            if m:
                assert hasattr(L, m.group(1)), m.group(1)


def test_library_loads_through_binding():
    _ensure_built()
    L = _lib.lib()
    assert b'commit_gb300' in L.cgb_version()
    assert L.cgb_last_error() is not None


def test_structs_match_header_layout():
    # field order/sizes of the ctypes mirrors (natural C alignment, LP64)
    assert ctypes.sizeof(_lib.CgbFistaParams) == 8 * 2 + 4 * 4 + 8 * 2 + 4 * 6  # 5 ints, padded to 8 bytes
    assert ctypes.sizeof(_lib.CgbFistaResult) == 8 * 7 + 4 * 6  # 5 ints, padded to 8 bytes
    assert _lib.CgbReg.coeff_weights.offset == 6 * 8 + 6 * 4 + 4 * 8
    assert _lib.CgbReg.level_ptr.offset == _lib.CgbReg.ngroups.offset + 8


def _sequential_group_prox(x, groups, w, lam):
    gidx = np.concatenate(groups).astype(np.int32)
    gsz = np.array([g.size for g in groups], np.int32)
    return O.prox_group_lasso(x.copy(), gidx, gsz, np.asarray(w, float), lam)


def _levelled_group_prox(x, groups, w, lam):
    """What the device does: groups of a level at once (all read before any write)."""
    order, lp = level_schedule(groups)
    x = x.copy()
    for k in range(lp.size - 1):
        lvl = [order[j] for j in range(lp[k], lp[k + 1])]
        norms = {g: np.linalg.norm(x[groups[g]]) for g in lvl}
        for g in lvl:
            idx = groups[g]
            wl = w[g] * lam
            if norms[g] <= wl:
                x[idx] = 0.0
            else:
                x[idx] *= (norms[g] - wl) / norms[g]
    return x


@pytest.mark.parametrize('seed', [0, 1, 2, 3])
def test_level_schedule_reproduces_sequential_group_prox(seed):
    rng = np.random.default_rng(seed)
    n = 60
    base = [np.sort(g) for g in np.array_split(rng.permutation(n), 6)]
    groups = [base[0], base[1], np.union1d(base[0], base[1]), base[2], base[3],
              np.union1d(base[2], base[3]), np.union1d(np.union1d(base[0], base[1]), base[2]), base[4], base[5]]
    if seed % 2:
        groups = groups[::-1]
    groups = [g.astype(np.int64) for g in groups]
    w = rng.uniform(0.5, 2.0, size=len(groups))
    x = rng.normal(size=n)
    order, lp = level_schedule(groups)
    # levels contain pairwise-disjoint groups
    for k in range(lp.size - 1):
        seen = set()
        for j in range(lp[k], lp[k + 1]):
            s = set(groups[order[j]].tolist())
            assert not (s & seen)
            seen |= s
    np.testing.assert_allclose(_levelled_group_prox(x, groups, w, 0.3), _sequential_group_prox(x, groups, w, 0.3),
                               rtol=1e-13, atol=1e-15)


def test_non_overlapping_groups_are_one_level():
    groups = [np.arange(i * 5, i * 5 + 5) for i in range(20)]
    order, lp = level_schedule(groups)
    assert lp.tolist() == [0, 20]


def test_regspec_reproduces_reference_flags():
    rp = O.reg_params({'IC': {'nSTR': 10}, 'EC': {'n': 4}, 'ISO': {'n': 3}},
                      {'wmr': np.zeros((1, 2, 3)), 'wmh': np.zeros((1, 2, 3)), 'iso': np.zeros((2, 3))})
    s = RegSpec(dict(rp))
    assert (s.sIC, s.nIC, s.sEC, s.nEC, s.sISO, s.nISO) == (0, 10, 10, 4, 14, 6)
    assert s.nn_ic and s.nn_ec and s.nn_iso
    rp2 = dict(rp, regIC='lasso', lambdaIC=0.5, nnIC=0)
    s2 = RegSpec(rp2)
    assert not s2.nn_ic and s2.lam_ic == 0.5


def test_product_package_never_uses_the_oracle():
    """The oracle is test infrastructure: nothing in the package imports, loads or runs it."""
    import glob
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for path in glob.glob(os.path.join(root, 'commit_gb300', '*.py')):
        src = open(path).read()
        for bad in ('import oracle', 'from oracle', "'oracle'", '"oracle"', 'trk2dict_oracle', 'commit_oracle',
                    'libcommit_ref', 'oracle/'):
            assert bad not in src, (path, bad)
