"""Oracle (test infrastructure only): FP64 NumPy restatement of the reference's gauge-invariant PEPS
for pure Z_N lattice gauge theory (phys_dim = 1), src/vmc/peps/gi/model.py and kernels.py.

Nothing here is imported by the product; the tests, ``__graft_entry__.smoke`` and ``bench.py``'s CPU
baseline use it as the checker.  Everything is batched over a leading sample axis z.

Model (model.py:41-119): site tensor A[r][c] has shape (1, nc, mu_u, mu_d, mu_l, mu_r) with
nc = N^(links - 1) gauge configurations and mu = dmax on interior bonds (equal degeneracies; the
uneven-degeneracy masks are not restated).  A sample is (sites, h_links, v_links) flattened
(model.py:121-144); the link values around a site select the slice A[r][c][0, cfg] (model.py:260-347)
and the amplitude is the standard boundary-MPS contraction of the selected slices.

The reference draws, per plaquette, delta = randint(1, N) and an accept uniform from split keys
(model.py:656-657, 682-683); here they are explicit arrays deltas[z, R-1, C-1] and
uniforms[z, R-1, C-1], as the standard engine takes explicit per-site uniforms.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .peps import (_ein, _left_update, _ones, apply_mpo_from_below, compute_right_envs, compute_right_envs_2row,
                   compute_single_gradient, contract_bottom, metropolis_ratio)

__all__ = ["GIConfig", "LinkDiagonalTerm", "PlaquetteTerm", "GIHamiltonian", "z2_pure_gauge_hamiltonian",
           "init_tensors", "flatten_sample", "unflatten_sample", "link_value", "site_cfg_index", "site_slices",
           "plaquette_flip", "random_physical_configuration", "amplitude", "init_cache", "transition",
           "estimate", "local_log_derivatives", "dense_hamiltonian_energy"]


@dataclass(frozen=True)
class GIConfig:
    """model.py:41-64 for pure gauge: phys_dim = 1, charge_of_site = (0,), Qx = 0."""
    shape: tuple
    N: int
    dmax: int


@dataclass(frozen=True)
class LinkDiagonalTerm:
    """gi/local_terms.py:12-39: sum over its links of diag[link value]."""
    orientation: str
    sites: tuple
    diag: np.ndarray


@dataclass(frozen=True)
class PlaquetteTerm:
    """local_terms.py:125-144."""
    row: int
    col: int
    coeff: float


@dataclass(frozen=True)
class GIHamiltonian:
    """gi/local_terms.py:63-77."""
    shape: tuple
    terms: tuple


def z2_pure_gauge_hamiltonian(shape, h=1.0, g=0.33, N=2):
    """examples/lgt/z2_pure_gauge.py:42-76 with gi/local_terms.py:80-90: -h (P + P^dag) per plaquette,
    g (2 - 2 cos(2 pi E / N)) per link."""
    R, C = shape
    diag = g * (2.0 - 2.0 * np.cos(2.0 * np.pi * np.arange(N) / N))
    terms = [PlaquetteTerm(r, c, -h) for r in range(R - 1) for c in range(C - 1)]
    terms += [LinkDiagonalTerm("h", ((r, c),), diag) for r in range(R) for c in range(C - 1)]
    terms += [LinkDiagonalTerm("v", ((r, c),), diag) for r in range(R - 1) for c in range(C)]
    return GIHamiltonian(tuple(shape), tuple(terms))


def _active(r, c, R, C):
    return {"left": c > 0, "right": c < C - 1, "up": r > 0, "down": r < R - 1}


def n_configs(cfg: GIConfig, r, c):
    """model.py:99-101."""
    R, C = cfg.shape
    links = sum(_active(r, c, R, C).values())
    return cfg.N ** max(links - 1, 0)


def bond_dims(cfg: GIConfig, r, c):
    """model.py:102-106: (mu_u, mu_d, mu_l, mu_r)."""
    R, C = cfg.shape
    return (cfg.dmax if r > 0 else 1, cfg.dmax if r < R - 1 else 1, cfg.dmax if c > 0 else 1,
            cfg.dmax if c < C - 1 else 1)


def init_tensors(cfg: GIConfig, seed=0, dtype=np.float64):
    """Seeded site tensors (1, nc, mu_u, mu_d, mu_l, mu_r), entries N(0,1)/sqrt(dmax^4)."""
    rng = np.random.default_rng(seed)
    R, C = cfg.shape
    out = []
    for r in range(R):
        row = []
        for c in range(C):
            shp = (1, n_configs(cfg, r, c)) + bond_dims(cfg, r, c)
            t = rng.standard_normal(shp) / np.sqrt(cfg.dmax ** 4)
            if np.issubdtype(np.dtype(dtype), np.complexfloating):
                t = (t + 1j * rng.standard_normal(shp) / np.sqrt(cfg.dmax ** 4)) / np.sqrt(2)
            row.append(t.astype(dtype))
        out.append(row)
    return out


def flatten_sample(sites, h, v):
    """model.py:121-129 (batched)."""
    z = sites.shape[0]
    return np.concatenate([sites.reshape(z, -1), h.reshape(z, -1), v.reshape(z, -1)], axis=1)


def unflatten_sample(sample, shape):
    """model.py:131-144 (batched)."""
    R, C = shape
    z = sample.shape[0]
    ns, nh = R * C, R * (C - 1)
    return (sample[:, :ns].reshape(z, R, C), sample[:, ns:ns + nh].reshape(z, R, C - 1),
            sample[:, ns + nh:].reshape(z, R - 1, C))


def link_value(h, v, r, c, direction):
    """model.py:221-257: the link on that side of site (r, c), 0 off the lattice."""
    z = h.shape[0]
    zero = np.zeros(z, dtype=np.int64)
    if direction == "left":
        return h[:, r, c - 1] if c > 0 else zero
    if direction == "right":
        return h[:, r, c] if c < h.shape[2] else zero
    if direction == "up":
        return v[:, r - 1, c] if r > 0 else zero
    if direction == "down":
        return v[:, r, c] if r < v.shape[1] else zero
    raise ValueError(direction)


def site_cfg_index(cfg: GIConfig, h, v, r, c):
    """model.py:308-347: base-N digits of the independent links in the order left, up, down, right;
    the first active of right, down, up, left is fixed by Gauss law and skipped."""
    R, C = cfg.shape
    active = _active(r, c, R, C)
    dependent = next((d for d in ("right", "down", "up", "left") if active[d]), None)
    idx = np.zeros(h.shape[0], dtype=np.int64)
    for d in ("left", "up", "down", "right"):
        if active[d] and d != dependent:
            idx = idx * cfg.N + link_value(h, v, r, c, d)
    return idx


def site_slices(cfg: GIConfig, h, v):
    """cfg index of every site, (z, R, C)."""
    R, C = cfg.shape
    return np.stack([np.stack([site_cfg_index(cfg, h, v, r, c) for c in range(C)], 1) for r in range(R)], 1)


def _site_mpo(tensors, cfg, h, v, r, c):
    """model.py:350-366 for one site: A[r][c][0, cfg] as (z, l, r, u, d)."""
    idx = site_cfg_index(cfg, h, v, r, c)
    return np.transpose(np.asarray(tensors[r][c])[0][idx], (0, 3, 4, 1, 2))


def row_mpo(tensors, cfg, h, v, row):
    return tuple(_site_mpo(tensors, cfg, h, v, row, c) for c in range(cfg.shape[1]))


def plaquette_flip(h, v, r, c, delta, N):
    """model.py:369-389 (batched over z with per-sample delta)."""
    h = h.copy()
    v = v.copy()
    h[:, r, c] = (h[:, r, c] + delta) % N
    h[:, r + 1, c] = (h[:, r + 1, c] - delta) % N
    v[:, r, c] = (v[:, r, c] + delta) % N
    v[:, r, c + 1] = (v[:, r, c + 1] - delta) % N
    return h, v


def random_physical_configuration(cfg: GIConfig, n, seed=0):
    """model.py:146-189 for pure gauge: random plaquette charges applied to the zero configuration."""
    rng = np.random.default_rng(seed)
    R, C = cfg.shape
    h = np.zeros((n, R, C - 1), dtype=np.int64)
    v = np.zeros((n, R - 1, C), dtype=np.int64)
    d = rng.integers(0, cfg.N, (n, R - 1, C - 1))
    h[:, :R - 1, :] += d
    h[:, 1:, :] -= d
    v[:, :, :C - 1] += d
    v[:, :, 1:] -= d
    return flatten_sample(np.zeros((n, R, C), dtype=np.int64), h % cfg.N, v % cfg.N)


def amplitude(tensors, cfg, samples, strategy):
    """Boundary-MPS amplitude of the selected slices (contraction.py:38-56)."""
    _, h, v = unflatten_sample(samples, cfg.shape)
    R, C = cfg.shape
    dtype = np.asarray(tensors[0][0]).dtype
    top = tuple(_ones(samples.shape[0], 3, dtype) for _ in range(C))
    for r in range(R):
        top = strategy.apply(top, row_mpo(tensors, cfg, h, v, r))
    return contract_bottom(top)


def init_cache(tensors, cfg, samples, strategy):
    """kernels.py:33-49 / model.py:881-898: bottom environments of every row."""
    _, h, v = unflatten_sample(samples, cfg.shape)
    R, C = cfg.shape
    dtype = np.asarray(tensors[0][0]).dtype
    envs = [None] * R
    env = tuple(_ones(samples.shape[0], 3, dtype) for _ in range(C))
    for r in range(R - 1, -1, -1):
        envs[r] = env
        env = apply_mpo_from_below(env, row_mpo(tensors, cfg, h, v, r), strategy)
    return envs


_PLAQ = "zalxe,zaub,zlruv,zxyvw,zewf,zbgc,zrsgh,zythi,zfij,zcstj->z"


def _plaquette_amp(left, top, bot, right_next, m00, m10, m01, m11, c):
    """model.py:656-666: the 2-row, 2-column amplitude with the given four site MPOs."""
    return np.einsum(_PLAQ, left, top[c], m00, m10, bot[c], top[c + 1], m01, m11, bot[c + 1], right_next,
                     optimize=True)


def _left2_update(left, top, m0, m1, bot):
    """model.py:695-699."""
    return _ein("zalxe,zaub,zlruv,zxyvw,zewf->zbryf", left, top, m0, m1, bot,
                path=[(0, 1), (0, 3), (0, 2), (0, 1)])


def _plaquette_sweep_row_pair(tensors, cfg, h, v, top, bottom, mpo0, mpo1, r, deltas, uniforms, margin):
    """model.py:629-703."""
    C = cfg.shape[1]
    dtype = mpo0[0].dtype
    z = h.shape[0]
    right = compute_right_envs_2row(top, mpo0, mpo1, bottom, dtype)
    left = _ones(z, 4, dtype)
    mpo0, mpo1 = list(mpo0), list(mpo1)
    for c in range(C - 1):
        delta = deltas[:, r, c]
        amp_cur = _plaquette_amp(left, top, bottom, right[c + 1], mpo0[c], mpo1[c], mpo0[c + 1], mpo1[c + 1], c)
        hp, vp = plaquette_flip(h, v, r, c, delta, cfg.N)
        m00 = _site_mpo(tensors, cfg, hp, vp, r, c)
        m01 = _site_mpo(tensors, cfg, hp, vp, r, c + 1)
        m10 = _site_mpo(tensors, cfg, hp, vp, r + 1, c)
        m11 = _site_mpo(tensors, cfg, hp, vp, r + 1, c + 1)
        amp_prop = _plaquette_amp(left, top, bottom, right[c + 1], m00, m10, m01, m11, c)
        ratio = metropolis_ratio(np.abs(amp_cur) ** 2, np.abs(amp_prop) ** 2)
        thr = np.minimum(1.0, ratio)
        u = uniforms[:, r, c]
        accept = u < thr
        margin[:] = np.minimum(margin, np.abs(thr - u))
        sel = accept.reshape((z,) + (1,) * 4)
        mpo0[c] = np.where(sel, m00, mpo0[c])
        mpo0[c + 1] = np.where(sel, m01, mpo0[c + 1])
        mpo1[c] = np.where(sel, m10, mpo1[c])
        mpo1[c + 1] = np.where(sel, m11, mpo1[c + 1])
        h = np.where(accept[:, None, None], hp, h)
        v = np.where(accept[:, None, None], vp, v)
        left = _left2_update(left, top[c], mpo0[c], mpo1[c], bottom[c])
    return tuple(mpo0), tuple(mpo1), h, v


def transition(tensors, cfg, samples, deltas, uniforms, bottom_envs, strategy):
    """model.py:901-1050, the phys_dim = 1 branch: plaquette sweeps over the row pairs.
    Returns (samples_next, amp, top_envs, margin), margin = min over plaquettes of |min(1, ratio) - u|."""
    sites, h, v = unflatten_sample(samples, cfg.shape)
    R, C = cfg.shape
    z = samples.shape[0]
    dtype = np.asarray(tensors[0][0]).dtype
    top_envs = [None] * R
    margin = np.full(z, np.inf)
    top = tuple(_ones(z, 3, dtype) for _ in range(C))
    mpo0 = row_mpo(tensors, cfg, h, v, 0)
    mpo1 = row_mpo(tensors, cfg, h, v, 1)
    for r in range(R - 1):
        top_envs[r] = top
        mpo0, mpo1, h, v = _plaquette_sweep_row_pair(tensors, cfg, h, v, top, bottom_envs[r + 1], mpo0, mpo1, r,
                                                     deltas, uniforms, margin)
        top = strategy.apply(top, mpo0)
        if r + 2 < R:
            mpo0 = mpo1
            mpo1 = row_mpo(tensors, cfg, h, v, r + 2)
    top_envs[R - 1] = top
    top = strategy.apply(top, mpo1)
    return flatten_sample(sites, h, v), contract_bottom(top), top_envs, margin


def estimate(tensors, cfg, samples, amp, operator, strategy, top_envs):
    """model.py:392-617 for pure gauge (link-diagonal and plaquette terms): env gradients of the
    selected slices, local energy, next bottom environments."""
    _, h, v = unflatten_sample(samples, cfg.shape)
    R, C = cfg.shape
    z = samples.shape[0]
    dtype = np.asarray(tensors[0][0]).dtype
    plaq = [[[] for _ in range(C - 1)] for _ in range(R - 1)]
    energy = np.zeros(z, dtype=np.result_type(amp.dtype, np.float64))
    for t in operator.terms:
        if isinstance(t, PlaquetteTerm):
            plaq[t.row][t.col].append(t)
        elif isinstance(t, LinkDiagonalTerm):
            links = h if t.orientation == "h" else v
            for rr, cc in t.sites:
                energy = energy + np.asarray(t.diag)[links[:, rr, cc]]
        else:
            raise NotImplementedError(f"{type(t).__name__} is not a pure-gauge term")
    grads = [[None] * C for _ in range(R)]
    bottom_cache = [None] * R
    bottom = tuple(_ones(z, 3, dtype) for _ in range(C))
    for row in range(R - 1, -1, -1):
        bottom_cache[row] = bottom
        top = top_envs[row]
        mpo = row_mpo(tensors, cfg, h, v, row)
        right = compute_right_envs(top, mpo, bottom, dtype)
        left = _ones(z, 3, dtype)
        for c in range(C):
            grads[row][c] = compute_single_gradient(left, right[c], top[c], bottom[c])
            left = _left_update(left, top[c], mpo[c], bottom[c])
        if row < R - 1 and any(plaq[row]):
            mpo_next = row_mpo(tensors, cfg, h, v, row + 1)
            bot_next = bottom_cache[row + 1]
            right2 = compute_right_envs_2row(top, mpo, mpo_next, bot_next, dtype)
            left2 = _ones(z, 4, dtype)
            for c in range(C - 1):
                if plaq[row][c]:
                    s = np.zeros(z, dtype=energy.dtype)
                    for delta in (1, -1):
                        hp, vp = plaquette_flip(h, v, row, c, np.full(z, delta), cfg.N)
                        s = s + _plaquette_amp(left2, top, bot_next, right2[c + 1],
                                               _site_mpo(tensors, cfg, hp, vp, row, c),
                                               _site_mpo(tensors, cfg, hp, vp, row + 1, c),
                                               _site_mpo(tensors, cfg, hp, vp, row, c + 1),
                                               _site_mpo(tensors, cfg, hp, vp, row + 1, c + 1), c)
                    coeff = sum(t.coeff for t in plaq[row][c])
                    energy = energy + coeff * s / amp
                left2 = _left2_update(left2, top[c], mpo[c], mpo_next[c], bot_next[c])
        bottom = apply_mpo_from_below(bottom, mpo, strategy)
    return grads, energy, bottom_cache


def local_log_derivatives(tensors, cfg, samples, grads, amp, full_gradient=False):
    """gi/kernels.py:78-120: sliced O (concatenated env gradients / amp) with the slice index
    sites * nc + cfg of every parameter, or the full gradient scattered at [site, cfg]."""
    _, h, v = unflatten_sample(samples, cfg.shape)
    R, C = cfg.shape
    z = samples.shape[0]
    parts, p = [], []
    for r in range(R):
        for c in range(C):
            g = grads[r][c].reshape(z, -1)
            idx = site_cfg_index(cfg, h, v, r, c)
            if full_gradient:
                t = np.asarray(tensors[r][c])
                full = np.zeros((z,) + t.shape, dtype=g.dtype)
                full[np.arange(z), 0, idx] = grads[r][c]
                parts.append(full.reshape(z, -1))
            else:
                parts.append(g)
                p.append(np.repeat(idx[:, None], g.shape[1], axis=1))
    o = np.concatenate(parts, axis=1) / amp[:, None]
    return o, (None if full_gradient else np.concatenate(p, axis=1))


def dense_hamiltonian_energy(tensors, cfg, operator, strategy):
    """Second oracle for small lattices: every gauge-invariant configuration (plaquette charges
    applied to the zero configuration), H in that basis (link-diagonal terms plus
    coeff (P + P^dag) between plaquette-flip neighbours), and E = <psi|H|psi> / <psi|psi>."""
    R, C = cfg.shape
    n_p = (R - 1) * (C - 1)
    charges = np.array(np.meshgrid(*([np.arange(cfg.N)] * n_p), indexing="ij")).reshape(n_p, -1).T
    n = charges.shape[0]
    h = np.zeros((n, R, C - 1), dtype=np.int64)
    v = np.zeros((n, R - 1, C), dtype=np.int64)
    for k in range(n_p):
        r, c = divmod(k, C - 1)
        h, v = plaquette_flip(h, v, r, c, charges[:, k], cfg.N)
    samples = flatten_sample(np.zeros((n, R, C), dtype=np.int64), h, v)
    psi = amplitude(tensors, cfg, samples, strategy)
    index = {tuple(s): i for i, s in enumerate(samples[:, R * C:])}
    H = np.zeros((n, n))
    for t in operator.terms:
        if isinstance(t, LinkDiagonalTerm):
            links = h if t.orientation == "h" else v
            for rr, cc in t.sites:
                H[np.arange(n), np.arange(n)] += np.asarray(t.diag)[links[:, rr, cc]]
        else:
            for delta in (1, -1):
                hp, vp = plaquette_flip(h, v, t.row, t.col, np.full(n, delta), cfg.N)
                tgt = [index[tuple(s)] for s in flatten_sample(np.zeros((n, R, C), dtype=np.int64), hp, vp)[:, R * C:]]
                H[np.arange(n), tgt] += t.coeff
    w = np.abs(psi) ** 2
    e_loc = (H @ psi) / psi
    return float(np.sum(w * e_loc.real) / np.sum(w)), samples, psi, e_loc
