"""Seeded synthetic COMMIT problems: tractogram -> dictionary, stick-zeppelin-ball LUTs, signal.

The reference builds its operator inputs from files written by ``trk2dictionary``
(commit/trk2dictionary/trk2dictionary_c.cpp:446-578, segments per (voxel, orientation))
and re-laid-out by ``Evaluation.load_dictionary`` (commit/core.pyx:436-582): segments are
stable-sorted by voxel (:508-514), lengths are divided by the fibre norm (:516-525) and
voxel ids are mapped to mask-voxel indices in Fortran order (:571-580).  Its LUTs come
from AMICO and are normalised per compartment (commit/core.pyx:411-431).

Neither the demo data nor AMICO is available, so this module generates stand-in inputs
with the same array shapes, dtypes and value ranges, from seeds:

* fibres are Catmull-Rom splines through 4-8 control points, sampled every 0.5 voxel;
  each step is assigned to the voxel of its midpoint (trk2dictionary splits steps at
  voxel faces instead, trk2dictionary_c.cpp:814-869) and to the nearest of ``ndirs``
  hemisphere directions; all steps of a fibre with equal (voxel, orientation) are
  merged by summing their lengths;
* EC peaks: 1-4 random orientations per fitted voxel; ISO: one element per voxel;
* LUTs: analytic stick (IC), zeppelin (EC) and ball (ISO) responses on a Fibonacci
  direction set, normalised like commit/core.pyx:411-431;
* x ~ U[0, 1], y = |A x + Rician noise| with sigma = 2 % of mean(A x).

Geometry uses seed ``seed``, x uses ``seed + 1`` and the noise ``seed + 2``.  The heavy
per-step arithmetic runs in torch on any device so the 1M-fibre workload can be built
on the GPU in seconds; all random draws come from numpy, so inputs do not depend on the
device beyond last-bit rounding of voxel/orientation assignment.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch


# --------------------------------------------------------------------------------------
# acquisition scheme and response functions
# --------------------------------------------------------------------------------------
def fibonacci_sphere(n: int, hemisphere: bool) -> np.ndarray:
    """n unit vectors spread on the sphere (or the z>=0 hemisphere) by a golden spiral."""
    i = np.arange(n, dtype=np.float64) + 0.5
    if hemisphere:
        z = 1.0 - i / n            # z in (0, 1]
    else:
        z = 1.0 - 2.0 * i / n      # z in (-1, 1)
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = i * math.pi * (3.0 - math.sqrt(5.0))
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def make_scheme(n_b0: int, shells: list[tuple[float, int]]) -> tuple[np.ndarray, np.ndarray]:
    """b-values [s/mm^2] and unit gradient directions for ``n_b0`` b0 plus the shells."""
    bvals = [np.zeros(n_b0)]
    bvecs = [np.zeros((n_b0, 3))]
    for k, (b, nd) in enumerate(shells):
        d = fibonacci_sphere(nd, hemisphere=False)
        # rotate each shell a little so the shells do not share directions
        a = 0.37 * (k + 1)
        rot = np.array([[math.cos(a), -math.sin(a), 0.0], [math.sin(a), math.cos(a), 0.0], [0.0, 0.0, 1.0]])
        bvals.append(np.full(nd, float(b)))
        bvecs.append(d @ rot.T)
    return np.concatenate(bvals), np.concatenate(bvecs)


def szb_kernels(bvals: np.ndarray, bvecs: np.ndarray, dirs: np.ndarray, d_par: float = 1.7e-3,
                d_perps: tuple = (0.51e-3,), d_isos: tuple = (1.7e-3, 3.0e-3),
                n_ic: int = 1, normalize: bool = True) -> dict:
    """Stick (IC), zeppelin (EC) and ball (ISO) LUTs, float32, shaped like AMICO's output.

    wmr: (n_ic, ndirs, nS), wmh: (len(d_perps), ndirs, nS), iso: (len(d_isos), nS).
    With n_ic > 1 the extra IC kernels use slightly smaller parallel diffusivities, the
    way multi-RF IC models do.  Normalisation follows commit/core.pyx:411-431: every
    kernel is divided by the norm of its first-direction response.
    """
    cos2 = (dirs @ bvecs.T) ** 2                                  # (ndirs, nS)
    b = bvals[None, :]
    wmr = np.stack([np.exp(-b * (d_par * (1.0 - 0.15 * i)) * cos2) for i in range(n_ic)])
    wmh = np.stack([np.exp(-b * (dp + (d_par - dp) * cos2)) for dp in d_perps]) if len(d_perps) else \
        np.zeros((0, dirs.shape[0], bvals.size))
    iso = np.stack([np.exp(-bvals * di) for di in d_isos]) if len(d_isos) else np.zeros((0, bvals.size))
    K = {'wmr': wmr.astype(np.float32), 'wmh': wmh.astype(np.float32), 'iso': iso.astype(np.float32)}
    if normalize:
        for key in ('wmr', 'wmh'):
            for i in range(K[key].shape[0]):
                K[key][i] /= np.float32(np.linalg.norm(K[key][i, 0, :]))
        for i in range(K['iso'].shape[0]):
            K['iso'][i] /= np.float32(np.linalg.norm(K['iso'][i]))
    for key in ('wmr', 'wmh', 'iso'):
        K[key] = np.ascontiguousarray(K[key], dtype=np.float32)
    return K


# --------------------------------------------------------------------------------------
# geometry
# --------------------------------------------------------------------------------------
def ellipsoid_mask(dim: tuple, n_vox: int) -> np.ndarray:
    """Boolean mask: the centred ellipsoid (axes proportional to dim) holding ~n_vox voxels."""
    g = np.stack(np.meshgrid(*[(np.arange(d) + 0.5 - d / 2.0) / (d / 2.0) for d in dim], indexing='ij'))
    r2 = (g ** 2).sum(0)
    if n_vox >= r2.size:
        return np.ones(dim, dtype=bool)
    thr = np.partition(r2.ravel(), n_vox - 1)[n_vox - 1]
    return r2 <= thr


def _ell_thr(dim: tuple, n_vox: int) -> float:
    g = np.stack(np.meshgrid(*[(np.arange(d) + 0.5 - d / 2.0) / (d / 2.0) for d in dim], indexing='ij'))
    r2 = (g ** 2).sum(0).ravel()
    return float(np.partition(r2, min(n_vox, r2.size) - 1)[min(n_vox, r2.size) - 1])


def _ell_r2(p: np.ndarray, dim: tuple, thr: float) -> np.ndarray:
    """Squared normalised radius of points p (m, 3) w.r.t. the mask ellipsoid (1 = surface)."""
    half = np.asarray(dim, dtype=np.float64) / 2.0
    return (((p - half) / half) ** 2).sum(1) / thr


def _catmull_rom(P: torch.Tensor, t: torch.Tensor) -> torch.Tensor:
    """Evaluate uniform Catmull-Rom pieces. P: (m, 4, 3) control points, t: (m,) in [0, 1]."""
    t = t[:, None]
    t2, t3 = t * t, t * t * t
    p0, p1, p2, p3 = P[:, 0], P[:, 1], P[:, 2], P[:, 3]
    return 0.5 * ((2 * p1) + (-p0 + p2) * t + (2 * p0 - 5 * p1 + 4 * p2 - p3) * t2 + (-p0 + 3 * p1 - 3 * p2 + p3) * t3)


@dataclass
class ProblemSpec:
    """Shape of one synthetic workload."""
    dim: tuple = (32, 32, 16)
    n_mask: int = 12000
    n_fibers: int = 5000
    ctrl: str = 'uniform'          # 'uniform' control points in the grid, or 'walk' with lognormal lengths
    mean_len: float = 120.0        # mean fibre length in voxels for ctrl='walk'
    step: float = 0.5
    ndirs: int = 500
    n_b0: int = 6
    shells: list = field(default_factory=lambda: [(1000.0, 60)])
    n_ic: int = 1
    d_perps: tuple = (0.51e-3,)
    d_isos: tuple = (1.7e-3, 3.0e-3)
    max_peaks: int = 4
    seed: int = 0


# named workloads (the reference's demo-scale case and the full-brain case)
SPECS = {
    # 32x32x16 grid, 12k-voxel mask, 5k splines through 4-8 uniform control points, nS=66
    'demo_5k': ProblemSpec(),
    # the demo case scaled to 50k streamlines (gradient checks)
    'demo_50k': ProblemSpec(n_fibers=50000),
    # 145x174x145 grid, 600k-voxel mask, 1M streamlines of lognormal length giving ~120
    # segments per streamline (arc length mean 86 voxels), 18 b0 + 3 shells x 90 dirs (nS=288)
    'hcp_1m': ProblemSpec(dim=(145, 174, 145), n_mask=600000, n_fibers=1000000, ctrl='walk',
                          mean_len=86.0, n_b0=18, shells=[(1000.0, 90), (2000.0, 90), (3000.0, 90)]),
}


# batched regularisation-path workload: 8 tractograms of uneven size on the full-brain grid
# and acquisition (seeds 10-17), each fitted for 16 lambda values log-spaced 1e-4..1e-1
# (fractions of lambda_max) with a nonnegative group lasso over 64 random bundles
BATCH_FIBERS = (50000, 100000, 150000, 200000, 250000, 300000, 350000, 400000)
BATCH_LAMBDAS = tuple(float(v) for v in np.logspace(-4, -1, 16))


def batch_spec(k: int, n_fibers: int | None = None) -> ProblemSpec:
    """Tractogram k (0-7) of the batched workload."""
    return scaled_spec('hcp_1m', n_fibers=int(n_fibers or BATCH_FIBERS[k]), seed=10 + k)


def bundle_groups(n_fibers: int, n_groups: int = 64, seed: int = 0) -> list:
    """A random partition of the streamlines into n_groups bundles (lists of IC columns)."""
    lab = np.random.default_rng(seed).integers(0, n_groups, size=n_fibers)
    return [np.flatnonzero(lab == g).astype(np.int64) for g in range(n_groups)]


def scaled_spec(name: str, **kw) -> ProblemSpec:
    s = SPECS[name]
    d = dict(s.__dict__)
    d.update(kw)
    return ProblemSpec(**d)


def _control_points(spec: ProblemSpec, rng: np.random.Generator, mask: np.ndarray):
    """Per-fibre control points (list of arrays) drawn from numpy only."""
    dim = np.array(spec.dim, dtype=np.float64)
    nf = spec.n_fibers
    nctrl = rng.integers(4, 9, size=nf)
    if spec.ctrl == 'uniform':
        pts = rng.uniform(0.0, 1.0, size=(int(nctrl.sum()), 3)) * dim
        return nctrl, pts
    # 'walk': start inside the mask, persistent random walk whose total length is lognormal
    sigma = 0.5
    mu = math.log(spec.mean_len) - 0.5 * sigma * sigma
    length = rng.lognormal(mu, sigma, size=nf)
    idx = np.flatnonzero(mask.ravel(order='F'))
    start = idx[rng.integers(0, idx.size, size=nf)]
    sx, sy, sz = np.unravel_index(start, spec.dim, order='F')
    p = np.stack([sx, sy, sz], 1).astype(np.float64) + rng.uniform(0, 1, size=(nf, 3))
    d = rng.normal(size=(nf, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    off = np.concatenate([[0], np.cumsum(nctrl)])
    pts = np.empty((int(off[-1]), 3))
    seglen = length / (nctrl - 1)
    maxk = int(nctrl.max())
    centre = dim / 2.0
    ell = _ell_thr(spec.dim, spec.n_mask)
    cur = p.copy()
    for k in range(maxk):
        live = nctrl > k
        pts[off[:-1][live] + k] = cur[live]
        nd = d + 0.6 * rng.normal(size=(nf, 3))
        nd /= np.linalg.norm(nd, axis=1, keepdims=True)
        d = nd
        nxt = cur + d * seglen[:, None]
        # keep the walk inside the mask ellipsoid: a step that would leave it is reflected
        # off the surface (specular reflection about the ellipsoid normal), and points are
        # pulled back onto the 0.9 level set if still outside
        out = _ell_r2(nxt, spec.dim, ell) > 0.9
        if out.any():
            nrm = (cur[out] - centre) / (centre ** 2)
            nrm /= np.linalg.norm(nrm, axis=1, keepdims=True) + 1e-12
            dd = d[out]
            dd = dd - 2.0 * np.sum(dd * nrm, axis=1, keepdims=True) * nrm
            d[out] = dd
            nxt[out] = cur[out] + dd * seglen[out, None]
        r2 = _ell_r2(nxt, spec.dim, ell)
        shrink = np.where(r2 > 0.9, np.sqrt(0.9 / np.maximum(r2, 1e-12)), 1.0)
        nxt = centre + (nxt - centre) * shrink[:, None]
        cur = np.clip(nxt, 0.0, dim - 1e-6)
    return nctrl, pts


def _voxelise(spec: ProblemSpec, nctrl: np.ndarray, pts: np.ndarray, dirs: np.ndarray,
              mask: np.ndarray, device: str, chunk: int = 200000):
    """Spline steps -> merged (fibre, voxel linear F-order index, orientation, length)."""
    dim = spec.dim
    dev = torch.device(device)
    dirs_t = torch.as_tensor(dirs, dtype=torch.float64, device=dev)
    mask_t = torch.as_tensor(mask.ravel(order='F'), dtype=torch.bool, device=dev)
    off = np.concatenate([[0], np.cumsum(nctrl)])
    out_f, out_v, out_o, out_l = [], [], [], []
    for c0 in range(0, spec.n_fibers, chunk):
        c1 = min(spec.n_fibers, c0 + chunk)
        P = torch.as_tensor(pts[off[c0]:off[c1]], dtype=torch.float64, device=dev)
        nc = torch.as_tensor(nctrl[c0:c1], dtype=torch.int64, device=dev)
        coff = torch.as_tensor(off[c0:c1 + 1] - off[c0], dtype=torch.int64, device=dev)
        nf = c1 - c0
        # pieces: fibre with k control points has k-1 pieces; pad ends by repetition
        npiece = nc - 1
        pfib = torch.repeat_interleave(torch.arange(nf, device=dev), npiece)
        pstart = torch.repeat_interleave(coff[:-1], npiece)
        pk = torch.arange(pfib.numel(), device=dev) - torch.repeat_interleave(torch.cumsum(npiece, 0) - npiece, npiece)
        last = torch.repeat_interleave(nc - 1, npiece)
        ids = torch.stack([pk - 1, pk, pk + 1, pk + 2], 1).clamp(min=0)
        ids = torch.minimum(ids, last[:, None]) + pstart[:, None]
        CP = P[ids]                                             # (npieces, 4, 3)
        chord = (CP[:, 2] - CP[:, 1]).norm(dim=1)
        nsteps = torch.clamp(torch.ceil(chord / spec.step), min=1).to(torch.int64)
        sp = torch.repeat_interleave(torch.arange(CP.shape[0], device=dev), nsteps + 1)
        sk = torch.arange(sp.numel(), device=dev) - torch.repeat_interleave(torch.cumsum(nsteps + 1, 0) - (nsteps + 1), nsteps + 1)
        t = sk.to(torch.float64) / nsteps[sp].to(torch.float64)
        X = _catmull_rom(CP[sp], t)                            # points, nsteps+1 per piece
        # consecutive points within a piece form steps
        valid = sk < nsteps[sp]
        a = X[:-1][valid[:-1]]
        b = X[1:][valid[:-1]]
        fib = pfib[sp[:-1][valid[:-1]]] + c0
        d = b - a
        ln = d.norm(dim=1)
        keep = ln > 0
        a, d, ln, fib = a[keep], d[keep], ln[keep], fib[keep]
        mid = a + 0.5 * d
        ijk = torch.floor(mid).to(torch.int64)
        inside = ((ijk >= 0) & (ijk < torch.tensor(dim, device=dev))).all(1)
        ijk, d, ln, fib = ijk[inside], d[inside], ln[inside], fib[inside]
        lin = ijk[:, 0] + dim[0] * (ijk[:, 1] + dim[1] * ijk[:, 2])
        inm = mask_t[lin]
        lin, d, ln, fib = lin[inm], d[inm], ln[inm], fib[inm]
        u = d / ln[:, None]
        o = torch.empty(u.shape[0], dtype=torch.int64, device=dev)
        for r0 in range(0, u.shape[0], 1 << 20):
            o[r0:r0 + (1 << 20)] = torch.argmax((u[r0:r0 + (1 << 20)] @ dirs_t.T).abs(), dim=1)
        # merge all steps of one fibre that share (voxel, orientation), summing their
        # lengths, as the per-fibre std::map of trk2dictionary_c.cpp:484-552 does
        if lin.numel():
            key = (fib * int(np.prod(dim)) + lin) * spec.ndirs + o
            ukey, inv = torch.unique(key, sorted=True, return_inverse=True)
            L = torch.zeros(ukey.numel(), dtype=torch.float64, device=dev).index_add_(0, inv, ln)
            uo = ukey % spec.ndirs
            rest = ukey // spec.ndirs
            ulin = rest % int(np.prod(dim))
            ufib = rest // int(np.prod(dim))
            out_f.append(ufib.cpu()); out_v.append(ulin.cpu())
            out_o.append(uo.cpu()); out_l.append(L.cpu())
    if not out_f:
        z = torch.zeros(0, dtype=torch.int64)
        return z, z, z, torch.zeros(0, dtype=torch.float64)
    return torch.cat(out_f), torch.cat(out_v), torch.cat(out_o), torch.cat(out_l)


def make_dictionary(spec: ProblemSpec, device: str = 'cpu') -> tuple[dict, dict]:
    """DICTIONARY and KERNELS dicts in the layout ``load_dictionary``/``load_kernels`` produce."""
    rng = np.random.default_rng(spec.seed)
    mask = ellipsoid_mask(spec.dim, spec.n_mask)
    dirs = fibonacci_sphere(spec.ndirs, hemisphere=True)
    bvals, bvecs = make_scheme(spec.n_b0, spec.shells)
    KERNELS = szb_kernels(bvals, bvecs, dirs, d_perps=spec.d_perps, d_isos=spec.d_isos, n_ic=spec.n_ic)

    nctrl, pts = _control_points(spec, rng, mask)
    f, lin, o, ln = _voxelise(spec, nctrl, pts, dirs, mask, device)
    f = f.numpy(); lin = lin.numpy(); o = o.numpy(); ln = ln.numpy()

    # fibres without segments are dropped and the rest renumbered (TRK kept flags)
    kept = np.zeros(spec.n_fibers, dtype=np.uint8)
    kept[np.unique(f)] = 1
    newid = np.cumsum(kept, dtype=np.int64) - 1
    f = newid[f]
    nSTR = int(kept.sum())
    norm = np.bincount(f, weights=ln, minlength=nSTR).astype(np.float32)

    # fitted voxels = voxels traversed by the tracts (the 'tdi' mask)
    tdi_lin = np.unique(lin)
    lut = np.full(int(np.prod(spec.dim)), -1, dtype=np.int64)
    lut[tdi_lin] = np.arange(tdi_lin.size)
    nV = int(tdi_lin.size)

    order = np.argsort(lin, kind='stable')
    IC = {
        'str': f[order].astype(np.uint32),
        'vox': lut[lin[order]].astype(np.uint32),
        'dir': o[order].astype(np.uint16),
        'len': ln[order].astype(np.float32),
    }
    IC['len'] = IC['len'] / norm[IC['str']]          # float32 division as commit/core.pyx:523-525
    IC['len'] = IC['len'].astype(np.float32)
    IC['n'] = int(IC['vox'].size)
    IC['nSTR'] = nSTR
    IC['nVOX'] = nV

    ec_n = rng.integers(1, spec.max_peaks + 1, size=nV) if spec.d_perps else np.zeros(nV, dtype=np.int64)
    ecv = np.repeat(np.arange(nV, dtype=np.uint32), ec_n)
    eco = rng.integers(0, spec.ndirs, size=ecv.size).astype(np.uint16)
    EC = {'vox': ecv, 'dir': eco, 'n': int(ecv.size)}
    ISO = {'vox': np.arange(nV, dtype=np.uint32), 'n': nV}

    tdi = np.zeros(int(np.prod(spec.dim)), dtype=np.uint8)
    tdi[tdi_lin] = 1
    DICTIONARY = {'IC': IC, 'EC': EC, 'ISO': ISO,
                  'TRK': {'kept': kept, 'norm': norm},
                  'ndirs': spec.ndirs, 'nV': nV, 'dim': spec.dim,
                  'MASK': tdi.reshape(spec.dim, order='F')}
    # mask voxel k sits at (MASK_ix[k], MASK_iy[k], MASK_iz[k]) (Fortran order, core.pyx:571-574)
    DICTIONARY['MASK_ix'], DICTIONARY['MASK_iy'], DICTIONARY['MASK_iz'] = np.unravel_index(tdi_lin, spec.dim, order='F')
    return DICTIONARY, KERNELS


def n_cols(D: dict, K: dict) -> int:
    return D['IC']['nSTR'] * K['wmr'].shape[0] + D['EC']['n'] * K['wmh'].shape[0] + D['ISO']['n'] * K['iso'].shape[0]


def n_rows(D: dict, K: dict) -> int:
    nS = K['wmr'].shape[2] if K['wmr'].size else (K['wmh'].shape[2] if K['wmh'].size else K['wmr'].shape[1])
    return D['IC']['nVOX'] * nS


def make_signal(Ax: np.ndarray, seed: int) -> np.ndarray:
    """y = |Ax + n| with Rician noise of sigma = 2 % of mean(Ax)."""
    rng = np.random.default_rng(seed)
    sigma = 0.02 * abs(float(np.mean(Ax)))
    n1 = rng.normal(0.0, sigma, size=Ax.shape)
    n2 = rng.normal(0.0, sigma, size=Ax.shape)
    return np.sqrt((Ax + n1) ** 2 + n2 ** 2)


def make_x(ncols: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).uniform(0.0, 1.0, size=ncols)


def voxel_slab(D: dict, K: dict, frac: float) -> dict:
    """A central slab of voxels holding about ``frac`` of the IC segments, as a dictionary of
    its own (voxels renumbered from 0, every streamline kept as a column, the slab's EC and
    ISO elements renumbered in voxel order).  The slab's operator is the restriction of A to
    the slab's rows: its A x is rows [lo*nS, hi*nS) of the full A x once x is mapped with
    ``cols`` (the full column of each slab column), and its A' y is the full A' of y zeroed
    outside those rows, read at ``cols``.  IC/EC/ISO arrays must be voxel-sorted, as
    load_dictionary leaves them (commit/core.pyx:508-562).

    Returns {'D': slab dictionary, 'share': its fraction of the IC segments, 'voxels':
    (lo, hi), 'cols': int64 array of full-column indices}."""
    vox = D['IC']['vox']
    nV = int(D['IC']['nVOX'])
    counts = np.bincount(vox, minlength=nV)
    c = np.cumsum(counts)
    n = int(c[-1])
    mid = int(np.searchsorted(c, n // 2))
    lo, hi = mid, mid
    target = max(1, int(frac * n))
    while (int(c[hi - 1]) if hi > 0 else 0) - (int(c[lo - 1]) if lo > 0 else 0) < target and (lo > 0 or hi < nV):
        lo = max(0, lo - max(1, (hi - lo) // 2 + 16))
        hi = min(nV, hi + max(1, (hi - lo) // 2 + 16))
    s0 = int(c[lo - 1]) if lo > 0 else 0
    s1 = int(c[hi - 1]) if hi > 0 else 0
    nIC, nEC, nISO = K['wmr'].shape[0], K['wmh'].shape[0], K['iso'].shape[0]
    IC = {k: np.ascontiguousarray(D['IC'][k][s0:s1]) for k in ('str', 'vox', 'dir', 'len')}
    IC['vox'] = (IC['vox'] - lo).astype(np.uint32)
    IC['n'] = s1 - s0
    IC['nSTR'] = D['IC']['nSTR']
    IC['nVOX'] = hi - lo
    ev = D['IC'].get('eval')
    IC['eval'] = np.ones(IC['nSTR'] * nIC, np.uint32) if ev is None else ev
    ecv = D['EC']['vox']
    e0, e1 = int(np.searchsorted(ecv, lo)), int(np.searchsorted(ecv, hi))
    EC = {'vox': (ecv[e0:e1] - lo).astype(np.uint32), 'dir': np.ascontiguousarray(D['EC']['dir'][e0:e1]),
          'n': e1 - e0}
    iv = D['ISO']['vox']
    i0, i1 = int(np.searchsorted(iv, lo)), int(np.searchsorted(iv, hi))
    ISO = {'vox': (iv[i0:i1] - lo).astype(np.uint32), 'n': i1 - i0}
    nF, nE, nI = int(D['IC']['nSTR']), int(D['EC']['n']), int(D['ISO']['n'])
    cols = [np.arange(nF * nIC, dtype=np.int64)]
    cols += [nF * nIC + i * nE + np.arange(e0, e1, dtype=np.int64) for i in range(nEC)]
    cols += [nF * nIC + nE * nEC + i * nI + np.arange(i0, i1, dtype=np.int64) for i in range(nISO)]
    return {'D': {'IC': IC, 'EC': EC, 'ISO': ISO}, 'share': (s1 - s0) / n if n else 0.0, 'voxels': (lo, hi),
            'cols': np.concatenate(cols)}
