"""CPU oracle for the FiRE local-energy hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import this module, and only as the checker.  The product path (``sparse_wf_gb300``)
never calls it.

Parity status: **parity unpinned**.  The reference (JAX/Flax/folx, Python only) cannot
be imported here (no jax/flax/folx) and ships no golden vectors for log|psi| or E_loc;
its tests are self-consistency tests only (sparse vs dense forward Laplacian,
``tests/test_fwd_lap.py:100-118``; low-rank vs full, ``tests/test_low_rank.py``).
This oracle is pinned the same way: its sparse forward Laplacian is checked against
finite differences of its own value path (``tests/test_oracle.py``).

What is restated (file:line in the reference project):

* neighbour lists ``get_pair_indices`` (``model/new_sparse_model.py:238-263``),
  ``get_neighbouring_nuclei`` (476-481), ``get_static_input`` (399-437), triplets
  ``_get_triplet_indices`` / ``_get_distinct_triplet_indices`` (``model/sparse_fwd_lap.py:228-291``);
* value path ``MoonLikeWaveFunction.signed`` (``model/wave_function.py:183-198``):
  ``NewSparseEmbedding.apply`` (``new_sparse_model.py:483-551``), ``Orbitals.__call__``
  (``model/orbitals.py:109-119``), ``signed_logpsi_from_orbitals`` (``model/utils.py:196-213``),
  ``Jastrow.__call__`` (``model/jastrow.py:261-307``);
* forward-Laplacian path ``_logpsi_with_fwd_lap_sparse`` (``wave_function.py:165-181``):
  ``apply_with_fwd_lap`` (``new_sparse_model.py:631-695``), ``contract_with_fwd_lap`` (95-131),
  ``NodeWithFwdLap`` and its ops (``sparse_fwd_lap.py:14-225, 322-335``), ``Orbitals.fwd_lap``
  (``orbitals.py:148-174``), ``sparse_slogdet_with_fwd_lap`` (``sparse_fwd_lap.py:294-319``),
  ``Jastrow.apply_with_fwd_lap`` (``jastrow.py:387-459``);
* ``kinetic_energy`` (``wave_function.py:215-221``), ``potential_energy``
  (``hamiltonian.py:15-26``), the all-electron Metropolis step (``mcmc.py:38-97``), the single-electron step
  (``mcmc.py:100-111, 196-275``), the jump to a nucleus (``mcmc.py:164-193``), the cluster update (``mcmc.py:119-161``) with
  externally supplied noise;
* the low-rank update of a cached state: ``log_psi_with_state`` / ``log_psi_low_rank_update``
  (``wave_function.py:226-287``), ``get_low_rank_pair_indices`` and ``NewSparseEmbedding.low_rank_update``
  (``new_sparse_model.py:414-474, 553-629``), ``Orbitals.low_rank_update`` (``orbitals.py:121-146``),
  ``woodburry_update`` (``model/utils.py:216-245``), ``Jastrow.low_rank_update`` (``jastrow.py:309-361``), driven by
  ``mcmc_steps_low_rank`` (``mcmc.py:196-275``); pinned like the reference's ``tests/test_low_rank.py:29-61``, against
  full evaluation;
* directional derivatives of log|psi| with respect to the parameters (``logpsi_jvp``, complex step): the checker of
  the per-walker parameter gradient that feeds SPRING (``preconditioner.py:118-262``).

folx (0.2.15, a dependency absent here) is replaced by ``FL``: a dense forward-mode
Laplacian carrier (value, Jacobian over T tangents, Laplacian), the published
forward-Laplacian algorithm (Li et al., 2023) -- for each primitive y = f(x):
J_y = f'(x) J_x and L_y = f'(x) L_x + f''(x) sum_t (J_x)_t^2, with the product rule for
bilinear ops.  Quirks of the reference that are reproduced on purpose:

1. ``SparseMLP`` applies bias AND SiLU on its last layer (``~is_last_layer`` on a Python bool
   is always truthy, ``sparse_fwd_lap.py:218-224``);
2. the neighbour list uses the raw cutoff, the e-e filter's cutoff function uses
   ``cutoff * sigmoid(cutoff_param)`` (``new_sparse_model.py:506, 644``);
3. padded nuclei sit at R = 1e6 with zero parameters (``new_sparse_model.py:481``);
4. ElElCusp sums i<j per spin block plus all up-down pairs (``utils.py:309-322``).
"""
from __future__ import annotations

import dataclasses

import numpy as np
import scipy.linalg
from scipy.special import expit

NO_NEIGHBOUR = 1_000_000  # model/graph_utils.py:14
FEATURE_DIM = 256
N_DET = 4
ATT_HEADS = 16
ATT_DIM = 16


# =============================================================================== scalar functions
# The value path also accepts complex parameters (the complex-step derivative of logpsi_jvp): for complex inputs
# these use analytic forms; real inputs take exactly the real code.
def sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x)) if np.iscomplexobj(x) else expit(x)


def softplus(x):
    if np.iscomplexobj(x):
        return np.where(x.real > 0, x + np.log1p(np.exp(-x)), np.log1p(np.exp(x)))
    return np.logaddexp(0.0, x)


def silu(x):
    return x * sigmoid(x)


def _log_abs(x):
    """log|x|; for complex x (a real value plus a complex-step perturbation) the analytic log(x sign(Re x))."""
    return np.log(x * np.sign(x.real)) if np.iscomplexobj(x) else np.log(np.abs(x))


def dsilu(x):
    s = expit(x)
    return s * (1.0 + x * (1.0 - s))


def d2silu(x):
    s = expit(x)
    return s * (1.0 - s) * (2.0 + x * (1.0 - 2.0 * s))


def cutoff_function(d, p=4):
    """``cutoff_function`` (``model/utils.py:103-112``): 1 + a d^p + b d^(p+1) + c d^(p+2) for d < 1."""
    a = -(p + 1) * (p + 2) * 0.5
    b = p * (p + 2)
    c = -p * (p + 1) * 0.5
    return np.where(np.real(d) < 1, 1 + a * d**p + b * d ** (p + 1) + c * d ** (p + 2), 0.0)


# =============================================================================== dense forward-Laplacian carrier
class FL:
    """x: value with shape S; j: Jacobian with shape (T,) + S; l: Laplacian with shape S."""

    __slots__ = ("x", "j", "l")
    __array_priority__ = 1000

    def __init__(self, x, j, l):
        self.x = np.asarray(x)
        self.j = np.asarray(j)
        self.l = np.asarray(l)

    @property
    def T(self):
        return self.j.shape[0]

    @property
    def shape(self):
        return self.x.shape

    @staticmethod
    def const(x, T):
        x = np.asarray(x)
        return FL(x, np.zeros((T,) + x.shape), np.zeros_like(x))

    def _bj(self, shape):
        return np.broadcast_to(self.j, (self.T,) + tuple(shape))

    def __add__(self, o):
        if isinstance(o, FL):
            x = self.x + o.x
            return FL(x, self._bj(x.shape) + o._bj(x.shape), self.l + o.l)
        x = self.x + o
        return FL(x, self._bj(x.shape), np.broadcast_to(self.l, x.shape))

    __radd__ = __add__

    def __neg__(self):
        return FL(-self.x, -self.j, -self.l)

    def __sub__(self, o):
        return self + (-o)

    def __rsub__(self, o):
        return (-self) + o

    def __mul__(self, o):
        if isinstance(o, FL):
            x = self.x * o.x
            j = self.j * o.x + self.x * o.j
            l = self.l * o.x + self.x * o.l + 2.0 * np.sum(self.j * o.j, axis=0)
            return FL(x, j, l)
        return FL(self.x * o, self.j * o, self.l * o)

    __rmul__ = __mul__

    def __truediv__(self, o):
        if isinstance(o, FL):
            return self * o.recip()
        return self * (1.0 / np.asarray(o))

    def ew(self, f, df, d2f):
        y, d1, d2 = f(self.x), df(self.x), d2f(self.x)
        return FL(y, self.j * d1, self.l * d1 + d2 * np.sum(self.j**2, axis=0))

    def lin(self, fn):
        """Apply a linear map (broadcasting over leading axes) to value, Jacobian and Laplacian."""
        return FL(fn(self.x), fn(self.j), fn(self.l))

    def matmul(self, W):
        return self.lin(lambda a: a @ W)

    def sum(self, axis):
        ax = axis % self.x.ndim
        return FL(self.x.sum(ax), self.j.sum(ax + 1), self.l.sum(ax))

    def __getitem__(self, idx):
        if not isinstance(idx, tuple):
            idx = (idx,)
        return FL(self.x[idx], self.j[(slice(None),) + idx], self.l[idx])

    def reshape(self, *shape):
        x = self.x.reshape(*shape)
        return FL(x, self.j.reshape((self.T,) + x.shape), self.l.reshape(x.shape))

    # primitives
    def exp(self):
        return self.ew(np.exp, np.exp, np.exp)

    def silu(self):
        return self.ew(silu, dsilu, d2silu)

    def log1p(self):
        return self.ew(np.log1p, lambda x: 1.0 / (1.0 + x), lambda x: -1.0 / (1.0 + x) ** 2)

    def log_abs(self):
        return self.ew(lambda x: np.log(np.abs(x)), lambda x: 1.0 / x, lambda x: -1.0 / x**2)

    def recip(self):
        return self.ew(lambda x: 1.0 / x, lambda x: -1.0 / x**2, lambda x: 2.0 / x**3)

    def sqrt(self):
        return self.ew(np.sqrt, lambda x: 0.5 / np.sqrt(x), lambda x: -0.25 * x ** (-1.5))

    def rsqrt(self):
        return self.ew(lambda x: x**-0.5, lambda x: -0.5 * x**-1.5, lambda x: 0.75 * x**-2.5)

    def cutoff(self):
        p = 4
        a, b, c = -(p + 1) * (p + 2) * 0.5, p * (p + 2), -p * (p + 1) * 0.5

        def f(d):
            return cutoff_function(d)

        def df(d):
            return np.where(d < 1, a * p * d ** (p - 1) + b * (p + 1) * d**p + c * (p + 2) * d ** (p + 1), 0.0)

        def d2f(d):
            return np.where(
                d < 1,
                a * p * (p - 1) * d ** (p - 2) + b * (p + 1) * p * d ** (p - 1) + c * (p + 2) * (p + 1) * d**p,
                0.0,
            )

        return self.ew(f, df, d2f)


def fl_concat(parts, axis):
    ax = axis % parts[0].x.ndim
    return FL(
        np.concatenate([p.x for p in parts], ax),
        np.concatenate([p.j for p in parts], ax + 1),
        np.concatenate([p.l for p in parts], ax),
    )


# =============================================================================== neighbour lists
def _pair_dist(r):
    """Pairwise distances with the rounding the device kernels use: ((dx^2 + dy^2) + dz^2), then sqrt.
    In float32 numpy rounds each product and sum (no fused multiply-add)."""
    d = r[:, None, :] - r[None, :, :]
    d2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    return np.sqrt(d2)


def in_cutoff_matrix(r, cutoff):
    """``is_neighbour`` (``model/graph_utils.py:179-184``): dist < cutoff, diagonal excluded."""
    r = np.asarray(r)
    dist = _pair_dist(r)
    np.fill_diagonal(dist, np.inf)
    return dist < np.asarray(cutoff, r.dtype)


def _where_padded(mask, size):
    rows, cols = np.nonzero(mask)  # row-major order, like jnp.where
    out_r = np.full(size, NO_NEIGHBOUR, np.int64)
    out_c = np.full(size, NO_NEIGHBOUR, np.int64)
    k = min(size, len(rows))
    out_r[:k] = rows[:k]
    out_c[:k] = cols[:k]
    return out_r, out_c


def pair_indices(r, n_up, cutoff, n_pairs_same=None, n_pairs_diff=None):
    """``get_pair_indices`` (``model/new_sparse_model.py:238-263``).

    Returns ((ct_same, nb_same, jac_same), (ct_diff, nb_diff, jac_diff), (jac_ctr, jac_dep)),
    all padded with NO_NEIGHBOUR to the requested sizes (defaults: exact counts)."""
    n = r.shape[0]
    spin = np.concatenate([np.zeros(n_up, bool), np.ones(n - n_up, bool)])
    inc = in_cutoff_matrix(r, cutoff)
    same = spin[:, None] == spin[None, :]
    if n_pairs_same is None:
        n_pairs_same = int(np.sum(inc & same))
    if n_pairs_diff is None:
        n_pairs_diff = int(np.sum(inc & ~same))
    ps = _where_padded(inc & same, n_pairs_same)
    pd = _where_padded(inc & ~same, n_pairs_diff)
    ct, nb = _where_padded(inc, n_pairs_same + n_pairs_diff)
    key = ct * n + nb
    jac_same = np.searchsorted(key, ps[0] * n + ps[1]) + n
    jac_diff = np.searchsorted(key, pd[0] * n + pd[1]) + n
    jac_ctr = np.concatenate([np.arange(n), ct])
    jac_dep = np.concatenate([np.arange(n), nb])
    return (ps[0], ps[1], jac_same), (pd[0], pd[1], jac_diff), (jac_ctr, jac_dep)


def en_dist(r, R):
    R = np.asarray(R, r.dtype)
    d = r[:, None, :] - R[None, :, :]
    return np.sqrt((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2])


def neighbouring_nuclei(r, R, cutoff_1el, n_neighbours_en):
    """``get_neighbouring_nuclei`` (``new_sparse_model.py:476-481``) for all electrons: [n, cap] indices."""
    inc = en_dist(r, R) < np.asarray(cutoff_1el, r.dtype)
    out = np.full((r.shape[0], n_neighbours_en), NO_NEIGHBOUR, np.int64)
    for i in range(r.shape[0]):
        idx = np.nonzero(inc[i])[0][:n_neighbours_en]
        out[i, : len(idx)] = idx
    return out


def static_counts(r, R, n_up, cutoff, cutoff_1el, laplacian=True):
    """``get_static_input`` without a move (``new_sparse_model.py:399-437``):
    (n_pairs_same, n_pairs_diff, n_triplets, n_neighbours_en)."""
    n = r.shape[0]
    spin = np.concatenate([np.zeros(n_up, bool), np.ones(n - n_up, bool)])
    inc = in_cutoff_matrix(r, cutoff)
    same = spin[:, None] == spin[None, :]
    n_en = int(np.max(np.sum(en_dist(r, R) < np.asarray(cutoff_1el, r.dtype), axis=-1)))
    deg = inc.sum(0).astype(np.int64)
    n_trip = int(np.sum(deg * deg)) if laplacian else 0
    return int(np.sum(inc & same)), int(np.sum(inc & ~same)), n_trip, n_en


def triplet_indices(jac_ctr, jac_dep, n_el, n_distinct_triplets):
    """``_get_triplet_indices`` (``model/sparse_fwd_lap.py:252-291``): (in, k, kn, i), same order."""
    P = len(jac_ctr) - n_el
    pi, pn = np.asarray(jac_ctr[n_el:]), np.asarray(jac_dep[n_el:])
    ar = np.arange(n_el)
    arP = np.arange(P) + n_el
    # distinct triplets: for every distinct pair (i, n) in order and every k ascending with (k, n) a pair
    keys = pi * n_el + pn
    t_in, t_k, t_kn, t_i = [], [], [], []
    for p in range(P):
        ks = np.arange(n_el)
        q = np.searchsorted(keys, ks * n_el + pn[p])
        qc = np.minimum(q, P - 1)
        ok = (q < P) & (pi[qc] == ks) & (pn[qc] == pn[p])
        sel = np.nonzero(ok)[0]
        t_in.append(np.full(len(sel), p))
        t_k.append(ks[sel])
        t_kn.append(qc[sel])
        t_i.append(np.full(len(sel), pi[p]))
    cat = (lambda a: np.concatenate(a) if a else np.zeros(0, np.int64))
    d_in, d_k, d_kn, d_i = cat(t_in), cat(t_k), cat(t_kn), cat(t_i)
    T = n_distinct_triplets
    pad = lambda a, fill: np.concatenate([a[:T], np.full(max(0, T - len(a)), fill, np.int64)])
    d_in = pad(d_in, NO_NEIGHBOUR // n_el)  # valid_trip_idx // n_el for the padding index
    d_k = pad(d_k, 0)
    d_kn = pad(d_kn, 0)
    d_i = pad(d_i, 0)
    trip_in = np.concatenate([ar, arP, pn, d_in + n_el])
    trip_k = np.concatenate([ar, pn, pi, d_k])
    trip_kn = np.concatenate([ar, pn, arP, d_kn + n_el])
    trip_i = np.concatenate([ar, pi, pn, d_i])
    return trip_in, trip_k, trip_kn, trip_i


# =============================================================================== value path
def _pairwise_filter_value(feat, kernel, bias, dir_W, dir_b, scales_raw, env_W, cutoff):
    """``PairwiseFilter`` (``model/utils.py:393-433``) on plain arrays; kernel/bias may be per-edge."""
    if kernel.ndim == 2:
        pre = feat @ kernel + bias
    else:
        pre = np.einsum("...k,...kf->...f", feat, kernel) + bias
    dirf = silu(pre) @ dir_W + dir_b
    dist = feat[..., 0]
    sc = softplus(scales_raw)
    env = np.exp(-((dist[..., None] / sc) ** 2)) * cutoff_function(dist / cutoff)[..., None]
    return dirf * (env @ env_W)


def _layer_norm(x, scale, bias, eps=1e-6):
    mu = x.mean(-1, keepdims=True)
    var = ((x - mu) ** 2).mean(-1, keepdims=True)
    return (x - mu) / np.sqrt(var + eps) * scale + bias


def elec_init_value(p, r, R, nb_idx, cutoff_1el):
    """ElecInit (``new_sparse_model.py:190-215``) for all electrons: returns [n, 5*F] pre-split output."""
    F = FEATURE_DIM
    Rp = np.concatenate([np.asarray(R, r.dtype), np.full((1, 3), 1e6, r.dtype)])
    idx = np.where(nb_idx == NO_NEIGHBOUR, len(R), nb_idx)
    pad = lambda a: np.concatenate([a, np.zeros((1,) + a.shape[1:], a.dtype)])
    Rn = Rp[idx]  # [n, E, 3]
    diff = r[:, None, :] - Rn
    dist = np.linalg.norm(diff, axis=-1, keepdims=True)
    feat = np.concatenate([dist, diff], -1)
    beta = _pairwise_filter_value(
        feat, pad(p["en_kernel"])[idx], pad(p["en_bias"])[idx], p["ei_dir_W"], p["ei_dir_b"],
        pad(p["en_scales"])[idx], p["ei_env_W"], cutoff_1el,
    )
    gamma = beta @ p["ei_gamma_W"]
    scaled = feat / feat[..., :1] * np.log1p(feat[..., :1])
    edge = scaled @ p["ei_edge_W"] + pad(p["en_nuc_emb"])[idx]
    h = np.einsum("neF,neF->nF", gamma, edge)
    h = _layer_norm(h, p["ei_ln_scale"], p["ei_ln_bias"])
    g = h @ p["ei_glu_W"]
    h = g[:, :F] * silu(g[:, F:])
    h = silu(h @ p["ei_dense_W"] + p["ei_dense_b"])
    return h @ p["ei_out_W"] + p["ei_out_b"]


def _edge_value(p, tag, rc, rn, cutoff_eff):
    diff = rc - rn
    dist = np.linalg.norm(diff, axis=-1, keepdims=True)
    feat = np.concatenate([dist, diff], -1)
    beta = _pairwise_filter_value(
        feat, p[f"ee{tag}_kernel"], p[f"ee{tag}_bias"], p[f"ee{tag}_dir_W"], p[f"ee{tag}_dir_b"],
        p[f"ee{tag}_scale"], p[f"ee{tag}_env_W"], cutoff_eff,
    )
    gamma = beta @ p[f"ee{tag}_gamma_W"]
    inp = feat / feat[..., :1] * np.log1p(feat[..., :1])
    return gamma, inp @ p[f"ee{tag}_edge_W"] + p[f"ee{tag}_edge_b"]


class Problem:
    """Molecule + architecture constants shared by the oracle entry points."""

    def __init__(self, R, Z, n_up, cutoff=5.0, cutoff_1el=20.0):
        self.R = np.asarray(R, np.float32)
        self.Z = np.asarray(Z, np.float64)
        self.n_el = int(np.sum(Z))
        self.n_up = int(n_up)
        self.n_nuc = len(self.Z)
        self.cutoff = float(cutoff)
        self.cutoff_1el = float(cutoff_1el)


def _contract(prob, p, r, ei, h, same_pairs, diff_pairs):
    """Adds the messages of the (center, neighbour) pairs to h in place, same-spin pairs first
    (``contract_pair``, ``new_sparse_model.py:82-93, 515-524``); ei is ElecInit's [n, 5F] output."""
    F = FEATURE_DIM
    _, ct_s, ct_d, nb_s, nb_d = (ei[:, k * F:(k + 1) * F] for k in range(5))
    cutoff_eff = prob.cutoff * sigmoid(p["cutoff_param"][0])
    for tag, (ct, nbi), mct, mnb in (("same", same_pairs, ct_s, nb_s), ("diff", diff_pairs, ct_d, nb_d)):
        if len(ct) == 0:
            continue
        gamma, edge = _edge_value(p, tag, r[ct], r[nbi], cutoff_eff)
        msg = gamma * silu(edge + mct[ct] + mnb[nbi])
        if np.iscomplexobj(msg) and not np.iscomplexobj(h):
            h = h.astype(msg.dtype)  # complex-step parameters of the e-e edges (logpsi_jvp)
        np.add.at(h, ct, msg)
    return h


def _node_update(p, h):
    """Per-electron update between the two stored normalisation scales (``new_sparse_model.py:525-528``)."""
    h = silu((h * p["scales"][0]) @ p["upd1_W"] + p["upd1_b"])
    h = silu(h @ p["upd2_W"] + p["upd2_b"])  # last-layer SiLU quirk (sparse_fwd_lap.py:218-224)
    return h * p["scales"][1]


def embedding_value(prob, p, r, return_pre_scale=False, return_init=False):
    """``NewSparseEmbedding.apply`` (``new_sparse_model.py:483-551``).  With ``return_init`` also returns
    ElecInit's [n, 5F] output (h0 and the four message maps, the embedding part of the low-rank state)."""
    F = FEATURE_DIM
    _, _, n_trip, n_en = static_counts(r32(r), prob.R, prob.n_up, prob.cutoff, prob.cutoff_1el, False)
    (cs, ns, _), (cd, nd, _), _ = pair_indices(r32(r), prob.n_up, prob.cutoff)
    nb = neighbouring_nuclei(r32(r), prob.R, prob.cutoff_1el, n_en)
    ei = elec_init_value(p, r, prob.R, nb, prob.cutoff_1el)
    h = _contract(prob, p, r, ei, ei[:, :F].copy(), (cs, ns), (cd, nd))
    if return_pre_scale:
        h_contract = h
        h = silu((h * p["scales"][0]) @ p["upd1_W"] + p["upd1_b"])
        return h_contract, silu(h @ p["upd2_W"] + p["upd2_b"])
    h = _node_update(p, h)
    return (h, ei) if return_init else h


def r32(r):
    """Neighbour lists are computed in the walkers' own dtype; the oracle's FP64 pass uses the
    float32 walkers for them so lists are bit-identical to the float32 device kernels."""
    return np.asarray(r, np.float32) if r.dtype == np.float64 else r


def _envelope_rows(prob, p, rs, spin):
    """Envelope rows [m, D*n] of electrons ``rs`` of one spin ("up" or "dn")."""
    d = np.linalg.norm(rs[:, None, :] - prob.R[None].astype(rs.dtype), axis=-1)  # [m, N]
    ex = np.exp(-d[:, :, None, None] * softplus(p[f"env_{spin}_sigma"])[None])  # [m, N, D, K]
    o = np.einsum("mNdk,Ndko->mdo", ex, p[f"env_{spin}_pi"])
    return o.reshape(len(rs), -1)


def envelopes_value(prob, p, r):
    """``EfficientIsotropicEnvelopes`` (``model/envelopes.py:55-82``) per spin: [n, D*n]."""
    nu = prob.n_up
    return np.concatenate([_envelope_rows(prob, p, r[:nu], "up"), _envelope_rows(prob, p, r[nu:], "dn")], 0)


def _orbital_rows(prob, p, h):
    """Raw orbital rows [n, D*n]: per-spin linear maps of the embeddings (``orbitals.py:109-115``)."""
    nu = prob.n_up
    return np.concatenate([h[:nu] @ p["orb_up_W"] + p["orb_up_b"], h[nu:] @ p["orb_dn_W"] + p["orb_dn_b"]], 0)


def _orbital_matrices(prob, raw, env):
    return (raw * env).reshape(prob.n_el, N_DET, prob.n_el).transpose(1, 0, 2)


def orbitals_value(prob, p, r, h):
    """``Orbitals.__call__`` (``model/orbitals.py:109-119``): [D, n, n]."""
    return _orbital_matrices(prob, _orbital_rows(prob, p, h), envelopes_value(prob, p, r))


def _spin_pair_dists(r, n_up):
    """``get_dist_same_diff`` (``model/utils.py:309-322``)."""
    d = np.linalg.norm(r[None, :, :] - r[:, None, :], axis=-1)
    iu = np.triu_indices(n_up, 1)
    same_up = d[:n_up, :n_up][iu]
    iu = np.triu_indices(len(r) - n_up, 1)
    same_dn = d[n_up:, n_up:][iu]
    return np.concatenate([same_up, same_dn]), d[:n_up, n_up:].reshape(-1)


def _jastrow_rows(p, h):
    """Per-electron Jastrow terms of embeddings h [m, F]: the MLP rows ``one_el`` [m, 2] (SparseMLP with final
    SiLU, ``jastrow.py:213-216, 363-364``), attention weights ``att`` [m, H] and weighted values ``vals``
    [m, H, A] (``jastrow.py:85-100``)."""
    q = (h @ p["att_Q_W"] + p["att_Q_b"]).reshape(-1, ATT_HEADS, ATT_DIM)
    v = (h @ p["att_V_W"] + p["att_V_b"]).reshape(-1, ATT_HEADS, ATT_DIM)
    att = np.exp(-(q * p["att_keys"]).sum(-1) / np.sqrt(ATT_DIM))
    vals = att[..., None] * v
    m = silu(h @ p["jmlp1_W"] + p["jmlp1_b"])
    m = silu(m @ p["jmlp2_W"] + p["jmlp2_b"])
    m = silu(m @ p["jmlp3_W"] + p["jmlp3_b"])
    one_el = m * p["mlp_scale"] + np.array([0.0, p["log_bias"][0]])
    return one_el, att, vals


def _jastrow_readout(prob, p, r, one_el, att, vals):
    """Cusp of r plus the attention readout (``jastrow.py:139-151``) and the summed MLP rows: (sign, log J)."""
    nu = prob.n_up
    a_s, a_d, f_s, f_d = p["cusp"]
    ds, dd = _spin_pair_dists(r, nu)
    logpsi = f_s * np.sum(a_s**2 / (a_s + ds)) + f_d * np.sum(a_d**2 / (a_d + dd))
    norm = np.stack([att[:nu].sum(0), att[nu:].sum(0)])
    vals = np.stack([vals[:nu].sum(0), vals[nu:].sum(0)])
    x = (vals / norm[..., None]).reshape(-1)
    x = silu(x @ p["att_out1_W"] + p["att_out1_b"])
    x = silu(x @ p["att_out2_W"] + p["att_out2_b"])
    x = x @ p["att_out3_W"] + p["att_out3_b"]
    J = x * p["att_scale"] + np.array([0.0, p["att_bias"][0]])
    J = J + one_el.sum(0)
    return np.sign(np.real(J[1])), logpsi + J[0] + _log_abs(J[1])


def jastrow_value(prob, p, r, h):
    """``Jastrow.__call__`` (``model/jastrow.py:261-307``) with psiformer cusp, MLP/log Jastrow and attention."""
    return _jastrow_readout(prob, p, r, *_jastrow_rows(p, h))


def logsumexp_signed(logdets, signs):
    m = np.max(np.real(logdets))
    s = np.sum(signs * np.exp(logdets - m))
    return np.sign(np.real(s)), m + _log_abs(s)


def slogdet_lu(A):
    """``slogdet_from_lu`` (``model/utils.py:153-161``) on a partial-pivoting LU."""
    lu, piv = scipy.linalg.lu_factor(A, check_finite=False)
    diag = np.diag(lu)
    parity = np.count_nonzero(piv != np.arange(len(piv))) + np.count_nonzero(np.real(diag) < 0)
    return (-1.0 if parity % 2 else 1.0), np.sum(_log_abs(diag)), (lu, piv)


def logpsi(prob, p, r):
    """(sign, log|psi|) of one walker: ``MoonLikeWaveFunction.signed`` (``wave_function.py:183-198``)."""
    h = embedding_value(prob, p, r)
    phi = orbitals_value(prob, p, r, h)
    sl = [slogdet_lu(phi[d])[:2] for d in range(N_DET)]
    s_det, l_det = logsumexp_signed(np.array([x[1] for x in sl]), np.array([x[0] for x in sl]))
    s_j, l_j = jastrow_value(prob, p, r, h)
    return s_det * s_j, l_det + l_j


def logpsi_jvp(prob, p, r, v, h=1e-30):
    """Directional derivative of log|psi| with respect to the parameters along v (a dict of arrays shaped like those
    of p; absent slots are zero), by the complex step: Im log|psi|(p + i h v) / h, exact to rounding because no two
    nearby values are subtracted (Squire and Trapp, SIAM Rev. 40, 1998).  It checks a per-walker parameter gradient g
    of log|psi| (the rows of SPRING's Jacobian, ``preconditioner.py:118-262``; ``update.py:177-191``) through
    <g, v> = logpsi_jvp(v) for any direction v."""
    pc = {k: (np.asarray(p[k], np.float64) + 1j * h * np.asarray(v[k], np.float64)) if k in v else p[k] for k in p}
    _, l = logpsi(prob, pc, np.asarray(r, np.float64))
    return float(np.imag(l)) / h


def potential_energy(r, R, Z):
    """``potential_energy`` (``hamiltonian.py:15-26``)."""
    r = np.asarray(r, np.float64)
    R = np.asarray(R, np.float64)
    Z = np.asarray(Z, np.float64)
    n = len(r)
    dee = np.linalg.norm(r[:, None] - r[None], axis=-1)
    iu = np.triu_indices(n, 1)
    e_ee = np.sum(1.0 / dee[iu])
    e_en = -np.sum(Z / np.linalg.norm(r[:, None] - R[None], axis=-1))
    dnn = np.linalg.norm(R[:, None] - R[None], axis=-1)
    iu = np.triu_indices(len(R), 1)
    e_nn = np.sum((Z[:, None] * Z[None])[iu] / dnn[iu])
    return e_ee + e_en + e_nn


# =============================================================================== sparse forward-Laplacian node
class SNode:
    """``NodeWithFwdLap`` (``model/sparse_fwd_lap.py:14-126``): x [n, ...], jac [n+P, 3, ...], lap [n, ...];
    jac rows: first the n self rows (dep == ctr), then one row per directed pair (ctr, dep)."""

    def __init__(self, x, jac, lap, idx_ctr, idx_dep):
        self.x, self.jac, self.lap = x, jac, lap
        self.idx_ctr, self.idx_dep = idx_ctr, idx_dep

    def _new(self, x, jac, lap):
        return SNode(x, jac, lap, self.idx_ctr, self.idx_dep)

    def linear(self, W, b=None):
        """``Linear`` (``sparse_fwd_lap.py:160-181``): bias on the value only."""
        y = self.x @ W
        if b is not None:
            y = y + b
        return self._new(y, self.jac @ W, self.lap @ W)

    def jac_sqr(self):
        """``get_jac_sqr`` (``sparse_fwd_lap.py:24-28``)."""
        out = np.zeros_like(self.x)
        np.add.at(out, self.idx_ctr, np.sum(self.jac**2, axis=1))
        return out

    def ew(self, f, df, d2f):
        """``ElementWise.apply_with_fwd_lap`` (``sparse_fwd_lap.py:196-206``)."""
        d1, d2 = df(self.x), d2f(self.x)
        return self._new(f(self.x), self.jac * d1[self.idx_ctr][:, None], self.lap * d1 + self.jac_sqr() * d2)

    def silu(self):
        return self.ew(silu, dsilu, d2silu)

    def scale(self, s):
        return self._new(self.x * s, self.jac * s, self.lap * s)

    def add_const(self, c):
        return self._new(self.x + c, self.jac, self.lap)

    def mul(self, o: "SNode"):
        """``NodeWithFwdLap.__mul__`` with another node of the same dependency structure (lines 87-96)."""
        y = self.x * o.x
        jac = self.jac * o.x[self.idx_ctr][:, None] + o.jac * self.x[self.idx_ctr][:, None]
        lap = self.lap * o.x + self.x * o.lap
        np.add.at(lap, self.idx_ctr, 2.0 * np.sum(self.jac * o.jac, axis=1))
        return self._new(y, jac, lap)

    def reshape(self, *shape):
        x = self.x.reshape(*shape)
        return self._new(x, self.jac.reshape(self.jac.shape[:2] + x.shape[1:]), self.lap.reshape(x.shape))

    def sum_last(self):
        return self._new(self.x.sum(-1), self.jac.sum(-1), self.lap.sum(-1))

    def expand_last(self):
        return self._new(self.x[..., None], self.jac[..., None], self.lap[..., None])

    def sum_over_nodes(self):
        """``sum_over_nodes`` (``sparse_fwd_lap.py:38-45``): FL with T = 3n (tangent = 3*dep + xyz)."""
        n = self.x.shape[0]
        jac = np.zeros((n, 3) + self.x.shape[1:])
        np.add.at(jac, self.idx_dep, self.jac)
        return FL(self.x.sum(0), jac.reshape((3 * n,) + self.x.shape[1:]), self.lap.sum(0))

    def sum_from_to(self, lo, hi):
        """``sum_from_to`` (``sparse_fwd_lap.py:47-56``)."""
        n = self.x.shape[0]
        mask = (self.idx_ctr >= lo) & (self.idx_ctr < hi)
        jac = np.zeros((n, 3) + self.x.shape[1:])
        np.add.at(jac, self.idx_dep[mask], self.jac[mask])
        return FL(self.x[lo:hi].sum(0), jac.reshape((3 * n,) + self.x.shape[1:]), self.lap[lo:hi].sum(0))


def _fl_electrons(r):
    """Per-electron 3-tangent carrier of the electron positions (the vmap'd folx input)."""
    n = r.shape[0]
    j = np.zeros((3, n, 3))
    for t in range(3):
        j[t, :, t] = 1.0
    return FL(r, j, np.zeros_like(r))


def _pairwise_filter_fl(feat: FL, kernel, bias, dir_W, dir_b, scales_raw, env_W, cutoff):
    if kernel.ndim == 2:
        pre = feat.matmul(kernel) + bias
    else:
        pre = feat.lin(lambda a: np.einsum("...k,...kf->...f", a, kernel)) + bias
    dirf = pre.silu().matmul(dir_W) + dir_b
    dist = feat[..., 0]
    sc = softplus(scales_raw)
    z = dist[..., None] * (1.0 / sc)
    env = (-(z * z)).exp() * (dist * (1.0 / cutoff)).cutoff()[..., None]
    return dirf * env.matmul(env_W)


def elec_init_fl(prob, p, r, nb_idx):
    """``jax.vmap(fwd_lap(h0_fn))`` (``new_sparse_model.py:648-650``): 5 FL outputs [n, F], T=3."""
    F = FEATURE_DIM
    R = prob.R.astype(r.dtype)
    Rp = np.concatenate([R, np.full((1, 3), 1e6)])
    idx = np.where(nb_idx == NO_NEIGHBOUR, len(R), nb_idx)
    pad = lambda a: np.concatenate([a, np.zeros((1,) + a.shape[1:])])
    re = _fl_electrons(r)
    diff = FL(re.x[:, None, :] - Rp[idx], np.broadcast_to(re.j[:, :, None, :], (3,) + idx.shape + (3,)),
              np.zeros(idx.shape + (3,)))
    dist = (diff * diff).sum(-1).sqrt()
    feat = fl_concat([dist[..., None], diff], -1)
    beta = _pairwise_filter_fl(feat, pad(p["en_kernel"])[idx], pad(p["en_bias"])[idx], p["ei_dir_W"],
                               p["ei_dir_b"], pad(p["en_scales"])[idx], p["ei_env_W"], prob.cutoff_1el)
    gamma = beta.matmul(p["ei_gamma_W"])
    d0 = feat[..., 0:1]
    scaled = feat * (d0.recip() * d0.log1p())
    edge = scaled.matmul(p["ei_edge_W"]) + pad(p["en_nuc_emb"])[idx]
    h = (gamma * edge).sum(1)
    # LayerNorm (flax, eps 1e-6)
    mu = h.sum(-1) * (1.0 / F)
    c = h - mu[:, None]
    var = (c * c).sum(-1) * (1.0 / F)
    inv = (var + 1e-6).rsqrt()
    h = c * inv[:, None] * p["ei_ln_scale"] + p["ei_ln_bias"]
    g = h.matmul(p["ei_glu_W"])
    h = g[:, :F] * g[:, F:].silu()
    h = (h.matmul(p["ei_dense_W"]) + p["ei_dense_b"]).silu()
    out = h.matmul(p["ei_out_W"]) + p["ei_out_b"]
    return [out[:, k * F:(k + 1) * F] for k in range(5)]


def _edge_fl(p, tag, rc, rn, cutoff_eff):
    P = rc.shape[0]
    jc = np.zeros((6, P, 3))
    jn = np.zeros((6, P, 3))
    for t in range(3):
        jc[t, :, t] = 1.0
        jn[t + 3, :, t] = 1.0
    diff = FL(rc - rn, jc - jn, np.zeros((P, 3)))
    dist = (diff * diff).sum(-1).sqrt()
    feat = fl_concat([dist[..., None], diff], -1)
    beta = _pairwise_filter_fl(feat, p[f"ee{tag}_kernel"], p[f"ee{tag}_bias"], p[f"ee{tag}_dir_W"],
                               p[f"ee{tag}_dir_b"], p[f"ee{tag}_scale"], p[f"ee{tag}_env_W"], cutoff_eff)
    gamma = beta.matmul(p[f"ee{tag}_gamma_W"])
    d0 = feat[..., 0:1]
    inp = feat * (d0.recip() * d0.log1p())
    edge = inp.matmul(p[f"ee{tag}_edge_W"]) + p[f"ee{tag}_edge_b"]
    return gamma, edge


def embedding_fl(prob, p, r):
    """``NewSparseEmbedding.apply_with_fwd_lap`` (``new_sparse_model.py:631-695``) -> SNode [n, F]."""
    n = prob.n_el
    rl = r32(r)
    _, _, _, n_en = static_counts(rl, prob.R, prob.n_up, prob.cutoff, prob.cutoff_1el, False)
    (cs, ns, js), (cd, nd, jd), (jac_ctr, jac_dep) = pair_indices(rl, prob.n_up, prob.cutoff)
    P = len(jac_ctr) - n
    nb = neighbouring_nuclei(rl, prob.R, prob.cutoff_1el, n_en)
    h0, ct_s, ct_d, nb_s, nb_d = elec_init_fl(prob, p, r, nb)
    cutoff_eff = prob.cutoff * sigmoid(p["cutoff_param"][0])
    x = h0.x.copy()
    lap = h0.l.copy()
    jac = np.zeros((n + P, 3, FEATURE_DIM))
    jac[:n] = h0.j.transpose(1, 0, 2)
    for tag, ct, nbi, jidx, mct, mnb in (("same", cs, ns, js, ct_s, nb_s), ("diff", cd, nd, jd, ct_d, nb_d)):
        if len(ct) == 0:
            continue
        gamma, edge = _edge_fl(p, tag, r[ct], r[nbi], cutoff_eff)
        zeros = np.zeros((3, len(ct), FEATURE_DIM))
        hc = FL(mct.x[ct], np.concatenate([mct.j[:, ct], zeros]), mct.l[ct])
        hn = FL(mnb.x[nbi], np.concatenate([zeros, mnb.j[:, nbi]]), mnb.l[nbi])
        msg = gamma * (edge + hc + hn).silu()
        np.add.at(x, ct, msg.x)
        np.add.at(lap, ct, msg.l)
        np.add.at(jac, ct, msg.j[:3].transpose(1, 0, 2))
        np.add.at(jac, jidx, msg.j[3:].transpose(1, 0, 2))
    h = SNode(x, jac, lap, jac_ctr, jac_dep)
    h = h.scale(p["scales"][0])
    h = h.linear(p["upd1_W"], p["upd1_b"]).silu()
    h = h.linear(p["upd2_W"], p["upd2_b"]).silu()
    return h.scale(p["scales"][1])


def envelopes_fl(prob, p, r):
    n, nu = prob.n_el, prob.n_up
    outs = []
    for spin, sl in (("up", slice(0, nu)), ("dn", slice(nu, n))):
        re = _fl_electrons(r[sl])
        R = prob.R.astype(np.float64)
        diff = FL(re.x[:, None, :] - R[None], np.broadcast_to(re.j[:, :, None, :], (3, re.x.shape[0], len(R), 3)),
                  np.zeros((re.x.shape[0], len(R), 3)))
        d = (diff * diff).sum(-1).sqrt()  # [m, N]
        sp = softplus(p[f"env_{spin}_sigma"])  # [N, D, K]
        ex = (d[:, :, None, None] * sp[None] * -1.0).exp()  # [m, N, D, K]
        pi = p[f"env_{spin}_pi"]
        o = ex.lin(lambda a: np.einsum("...mNdk,Ndko->...mdo", a, pi))
        outs.append(o.reshape(re.x.shape[0], -1))
    return fl_concat(outs, 0)


def orbitals_fl(prob, p, r, h: SNode):
    """``Orbitals.fwd_lap`` sparse branch (``orbitals.py:148-174``) -> per-det x [D,n,n], jac [D,n+P,3,n], lap."""
    n, nu = prob.n_el, prob.n_up
    up = h.linear(p["orb_up_W"], p["orb_up_b"])
    dn = h.linear(p["orb_dn_W"], p["orb_dn_b"])
    # merge_up_down (sparse_fwd_lap.py:129-137)
    x = np.concatenate([up.x[:nu], dn.x[nu:]])
    lap = np.concatenate([up.lap[:nu], dn.lap[nu:]])
    jac = np.where((h.idx_ctr < nu)[:, None, None], up.jac, dn.jac)
    env = envelopes_fl(prob, p, r)
    # multiply_with_1el_fn (sparse_fwd_lap.py:322-335)
    jb = env.j.transpose(1, 0, 2)  # [n, 3, C]
    out = x * env.x
    jac_out = np.zeros_like(jac)
    jac_out[:n] = x[:, None, :] * jb + env.x[:, None, :] * jac[:n]
    jac_out[n:] = env.x[h.idx_ctr[n:]][:, None, :] * jac[n:]
    lap_out = lap * env.x + env.l * x + 2.0 * np.sum(jac[:n] * jb, axis=1)
    D = N_DET
    phi = out.reshape(n, D, n).transpose(1, 0, 2)
    lp = lap_out.reshape(n, D, n).transpose(1, 0, 2)
    jc = jac_out.reshape(jac_out.shape[0], 3, D, n).transpose(2, 0, 1, 3)
    return phi, jc, lp


def sparse_slogdet_fl(A, jac, lap, idx_ctr, idx_dep, n_triplets):
    """``sparse_slogdet_with_fwd_lap`` (``sparse_fwd_lap.py:294-319``): (sign, logdet, jac[3n], lap)."""
    n = A.shape[0]
    sign, logdet, (lu, piv) = slogdet_lu(A)
    Ainv = scipy.linalg.lu_solve((lu, piv), np.eye(n), check_finite=False)
    M = jac @ Ainv  # [n+P, 3, n]
    nP = len(idx_ctr)
    jl = np.zeros((n, 3))
    np.add.at(jl, idx_dep, M[np.arange(nP), :, idx_ctr])
    t_in, t_k, t_kn, t_i = triplet_indices(idx_ctr, idx_dep, n, n_triplets)
    ll = np.einsum("ij,ji", lap, Ainv) - np.sum(M[t_in, :, t_k] * M[t_kn, :, t_i])
    return sign, logdet, jl.reshape(-1), ll


def cusp_fl(prob, p, r):
    """Analytic forward Laplacian of ``ElElCusp`` (``jastrow.py:48-64``): value, grad [3n], Laplacian."""
    n, nu = prob.n_el, prob.n_up
    a_s, a_d, f_s, f_d = p["cusp"]
    diff = r[:, None, :] - r[None, :, :]
    d = np.linalg.norm(diff, axis=-1)
    np.fill_diagonal(d, 1.0)
    spin = np.arange(n) < nu
    same = spin[:, None] == spin[None, :]
    alpha = np.where(same, a_s, a_d)
    fac = np.where(same, f_s, f_d)
    u = alpha**2 / (alpha + d)
    du = -(alpha**2) / (alpha + d) ** 2
    d2u = 2 * alpha**2 / (alpha + d) ** 3
    off = ~np.eye(n, dtype=bool)
    val = 0.5 * np.sum((fac * u)[off])
    g = np.where(off[..., None], (fac * du / d)[..., None] * diff, 0.0).sum(1)  # [n, 3]
    lap = np.sum(np.where(off, fac * (d2u + 2 * du / d), 0.0))
    return val, g.reshape(-1), lap


def jastrow_fl(prob, p, r, h: SNode):
    """``Jastrow.apply_with_fwd_lap`` (``jastrow.py:387-459``) -> (value, jac [3n], lap)."""
    nu, n = prob.n_up, prob.n_el
    cv, cg, cl = cusp_fl(prob, p, r)
    # attention on the sparse node (jastrow.py:434-440, 85-100, 132-137)
    q = h.linear(p["att_Q_W"], p["att_Q_b"]).reshape(n, ATT_HEADS, ATT_DIM)
    keys = p["att_keys"]
    att = SNode(q.x * keys, q.jac * keys, q.lap * keys, q.idx_ctr, q.idx_dep).sum_last()
    s = 1.0 / np.sqrt(ATT_DIM)
    att = att.ew(lambda x: np.exp(-x * s), lambda x: -s * np.exp(-x * s), lambda x: s * s * np.exp(-x * s))
    v = h.linear(p["att_V_W"], p["att_V_b"]).reshape(n, ATT_HEADS, ATT_DIM)
    vals = att.expand_last().mul(v)
    up_n, dn_n = att.sum_from_to(0, nu), att.sum_from_to(nu, n)
    up_v, dn_v = vals.sum_from_to(0, nu), vals.sum_from_to(nu, n)
    stack = lambda a, b: FL(np.stack([a.x, b.x]), np.stack([a.j, b.j], 1), np.stack([a.l, b.l]))
    norm, values = stack(up_n, dn_n), stack(up_v, dn_v)
    x = (values / norm[..., None]).reshape(-1)
    x = (x.matmul(p["att_out1_W"]) + p["att_out1_b"]).silu()
    x = (x.matmul(p["att_out2_W"]) + p["att_out2_b"]).silu()
    x = x.matmul(p["att_out3_W"]) + p["att_out3_b"]
    J = x * p["att_scale"] + np.array([0.0, p["att_bias"][0]])
    # MLP Jastrow (SparseMLP with final SiLU) + sum_over_nodes (jastrow.py:451-455)
    m = h.linear(p["jmlp1_W"], p["jmlp1_b"]).silu()
    m = m.linear(p["jmlp2_W"], p["jmlp2_b"]).silu()
    m = m.linear(p["jmlp3_W"], p["jmlp3_b"]).silu()
    m = m.scale(p["mlp_scale"]).add_const(np.array([0.0, p["log_bias"][0]]))
    J = J + m.sum_over_nodes()
    lj = J[0] + J[1].log_abs()
    return cv + lj.x, cg + lj.j, cl + lj.l


def logpsi_fl(prob, p, r):
    """``_logpsi_with_fwd_lap_sparse`` (``wave_function.py:165-181``) -> (log|psi|, jac [3n], lap)."""
    n = prob.n_el
    h = embedding_fl(prob, p, r)
    phi, jac, lap = orbitals_fl(prob, p, r, h)
    _, _, n_trip, _ = static_counts(r32(r), prob.R, prob.n_up, prob.cutoff, prob.cutoff_1el)
    res = [sparse_slogdet_fl(phi[d], jac[d], lap[d], h.idx_ctr, h.idx_dep, n_trip) for d in range(N_DET)]
    signs = np.array([x[0] for x in res])
    ld = FL(np.array([x[1] for x in res]), np.stack([x[2] for x in res], 1), np.array([x[3] for x in res]))
    m = np.max(ld.x)
    w = (ld + (-m)).exp() * signs
    lse = w.sum(0).log_abs() + m
    jv, jj, jl = jastrow_fl(prob, p, r, h)
    return lse.x + jv, lse.j + jj, lse.l + jl


def kinetic_energy(prob, p, r):
    """``MoonLikeWaveFunction.kinetic_energy`` (``wave_function.py:215-221``)."""
    _, j, l = logpsi_fl(prob, p, r)
    return -0.5 * (l + np.dot(j, j))


def local_energy(prob, p, r):
    """``local_energy`` (``hamiltonian.py:69-81``) without pseudopotentials."""
    return kinetic_energy(prob, p, r) + potential_energy(r, prob.R, prob.Z)


def woodbury_update(sign, logdet, A, Ainv, A_new, changed):
    """``woodburry_update`` (``model/utils.py:216-245``): rows ``changed`` of A are replaced by those of A_new.
    Matrix determinant lemma for the slogdet, det(A') = det(A) det(I + V A^-1[:, changed]) with V the row changes,
    and the Woodbury identity for the inverse.  Indices outside [0, n) (NO_NEIGHBOUR padding of cluster moves)
    contribute nothing, as the reference's ``mode="fill"`` gathers do.  Returns ((sign', logdet'), A'^-1)."""
    n = A.shape[0]
    changed = np.asarray(changed)
    ok = (changed >= 0) & (changed < n)
    safe = np.where(ok, changed, 0)
    V = np.where(ok[:, None], A_new[safe] - A[safe], 0.0)          # [k, n]
    AinvU = np.where(ok[None, :], Ainv[:, safe], 0.0)              # [n, k]
    M = np.eye(len(changed)) + V @ AinvU
    s_d, l_d = np.linalg.slogdet(M)
    new_inv = Ainv - AinvU @ np.linalg.inv(M) @ V @ Ainv
    return (sign * s_d, logdet + l_d), new_inv


# =============================================================================== low-rank update
@dataclasses.dataclass
class LowRankState:
    """``LowRankState`` (``model/wave_function.py:226-247``) of one walker: what a move of a few electrons reuses.

    r [n, 3]; ei [n, 5F] ElecInit output (h0 | msg_ct_same | msg_ct_diff | msg_nb_same | msg_nb_diff,
    ``EmbeddingState``); h [n, F] embeddings; env, orb [n, D n] envelope and raw orbital rows (``OrbitalState``);
    A, Ainv [D, n, n], signs, logdets [D] (``LogPsiState``); one_el [n, 2], att [n, H], vals [n, H, A]
    (``JastrowState``)."""

    r: np.ndarray
    ei: np.ndarray
    h: np.ndarray
    env: np.ndarray
    orb: np.ndarray
    A: np.ndarray
    Ainv: np.ndarray
    signs: np.ndarray
    logdets: np.ndarray
    one_el: np.ndarray
    att: np.ndarray
    vals: np.ndarray


def _moved(n, idx_changed):
    """In-range moved electrons.  Padded entries (NO_NEIGHBOUR, from cluster moves) gather electron n - 1, as an
    out-of-range JAX gather clamps, and are dropped by scatters."""
    idx = np.asarray(idx_changed, np.int64)
    return idx[(idx >= 0) & (idx < n)], np.clip(idx, 0, n - 1)


def affected_electrons(prob, r_old, r_new, idx_changed):
    """Electrons whose embedding changes when ``idx_changed`` move from r_old to r_new, and the pairs needed to
    recompute them (``get_low_rank_pair_indices``, ``new_sparse_model.py:439-474``): every electron within the
    cutoff of a moved electron before or after the move, plus the moved ones.  Returns (mask [n], required [n, n])
    with required[i, j] = i affected and j a neighbour of i after the move."""
    n = prob.n_el
    moved, gathered = _moved(n, idx_changed)
    inc_old = in_cutoff_matrix(r32(r_old), prob.cutoff)
    inc_new = in_cutoff_matrix(r32(r_new), prob.cutoff)
    aff = np.any(inc_old[:, gathered] | inc_new[:, gathered], axis=-1)
    aff[moved] = True
    return aff, inc_new & aff[:, None]


def changed_counts(prob, r_old, r_new, idx_changed):
    """The move statics of ``get_static_input`` (``new_sparse_model.py:414-424``):
    (n_changed_hout, n_changed_pair_same, n_changed_pair_diff)."""
    aff, req = affected_electrons(prob, r_old, r_new, idx_changed)
    spin = np.arange(prob.n_el) < prob.n_up
    same = spin[:, None] == spin[None, :]
    return int(aff.sum()), int(np.sum(req & same)), int(np.sum(req & ~same))


def logpsi_with_state(prob, p, r):
    """``log_psi_with_state`` (``wave_function.py:226-247``): ((sign, log|psi|), LowRankState); the inverses
    come from an LU (``slog_and_inverse``, ``model/utils.py:164-175``)."""
    h, ei = embedding_value(prob, p, r, return_init=True)
    env = envelopes_value(prob, p, r)
    orb = _orbital_rows(prob, p, h)
    A = _orbital_matrices(prob, orb, env)
    sl = [slogdet_lu(A[d]) for d in range(N_DET)]
    Ainv = np.stack([scipy.linalg.lu_solve(x[2], np.eye(prob.n_el)) for x in sl])
    one_el, att, vals = _jastrow_rows(p, h)
    st = LowRankState(r.copy(), ei, h, env, orb, A, Ainv, np.array([x[0] for x in sl]),
                      np.array([x[1] for x in sl]), one_el, att, vals)
    s_det, l_det = logsumexp_signed(st.logdets, st.signs)
    s_j, l_j = _jastrow_readout(prob, p, r, one_el, att, vals)
    return (s_det * s_j, l_det + l_j), st


def logpsi_low_rank_update(prob, p, r, idx_changed, state):
    """``log_psi_low_rank_update`` (``wave_function.py:249-287``): log|psi| at r, where only electrons
    ``idx_changed`` moved since ``state``, from recomputed rows only.

    * embedding (``NewSparseEmbedding.low_rank_update``, ``new_sparse_model.py:553-629``): ElecInit rows of the moved
      electrons; every affected electron is reset to h0 and its messages are contracted again over its neighbours
      after the move, then updated;
    * orbitals (``Orbitals.low_rank_update``, ``orbitals.py:121-146``): envelope rows of the moved electrons, raw
      orbital rows of the affected ones;
    * determinants (``signed_log_psi_from_orbitals_low_rank``, ``model/utils.py:287-306``): the determinant lemma
      and the Woodbury update of A^-1 over the affected rows;
    * Jastrow (``Jastrow.low_rank_update``, ``jastrow.py:309-361``): MLP and attention rows of the affected
      electrons, the cusp in full.

    Returns ((sign, log|psi|), LowRankState at r)."""
    F = FEATURE_DIM
    n, nu = prob.n_el, prob.n_up
    moved, _ = _moved(n, idx_changed)
    aff, req = affected_electrons(prob, state.r, r, idx_changed)
    rows = np.nonzero(aff)[0]
    spin = np.arange(n) < nu
    same = spin[:, None] == spin[None, :]

    ei = state.ei.copy()
    if len(moved):
        n_en = static_counts(r32(r), prob.R, nu, prob.cutoff, prob.cutoff_1el, False)[3]
        nb = neighbouring_nuclei(r32(r)[moved], prob.R, prob.cutoff_1el, n_en)
        ei[moved] = elec_init_value(p, r[moved], prob.R, nb, prob.cutoff_1el)
    h = state.h.copy()
    h[rows] = ei[rows, :F]
    h = _contract(prob, p, r, ei, h, np.nonzero(req & same), np.nonzero(req & ~same))
    h[rows] = _node_update(p, h[rows])

    env = state.env.copy()
    for sp, sel in (("up", moved[moved < nu]), ("dn", moved[moved >= nu])):
        if len(sel):
            env[sel] = _envelope_rows(prob, p, r[sel], sp)
    orb = state.orb.copy()
    up, dn = rows[rows < nu], rows[rows >= nu]
    orb[up] = h[up] @ p["orb_up_W"] + p["orb_up_b"]
    orb[dn] = h[dn] @ p["orb_dn_W"] + p["orb_dn_b"]
    A = _orbital_matrices(prob, orb, env)
    signs, logdets, Ainv = state.signs.copy(), state.logdets.copy(), np.empty_like(state.Ainv)
    for d in range(N_DET):
        (signs[d], logdets[d]), Ainv[d] = woodbury_update(state.signs[d], state.logdets[d], state.A[d],
                                                          state.Ainv[d], A[d], rows)

    one_el, att, vals = state.one_el.copy(), state.att.copy(), state.vals.copy()
    if len(rows):
        one_el[rows], att[rows], vals[rows] = _jastrow_rows(p, h[rows])
    st = LowRankState(r.copy(), ei, h, env, orb, A, Ainv, signs, logdets, one_el, att, vals)
    s_det, l_det = logsumexp_signed(logdets, signs)
    s_j, l_j = _jastrow_readout(prob, p, r, one_el, att, vals)
    return (s_det * s_j, l_det + l_j), st


def mcmc_block(prob, p, r, noise, log_u, width):
    """All-electron Metropolis block (``mcmc.py:38-97``) with externally supplied draws.

    noise [steps, n, 3] ~ N(0, 1), log_u [steps] = log U(0, 1).  Returns (r, log_prob, n_accept, margins)
    where margins[s] = log_ratio - log_u (accept iff > 0)."""
    lp = 2.0 * logpsi(prob, p, r)[1]
    n_acc = 0
    margins = []
    for s in range(noise.shape[0]):
        rn = r + noise[s] * width
        lpn = 2.0 * logpsi(prob, p, rn)[1]
        m = (lpn - lp) - log_u[s]
        margins.append(m)
        if m > 0:
            r, lp = rn, lpn
            n_acc += 1
    return r, lp, n_acc, np.array(margins)


def jump_proposal(R, Z, r, d, sigma):
    """``proposal_jump_to_atom`` (``mcmc.py:164-193``) for draws d = (u_electron, u_nucleus, eps[3]): electron
    min(floor(u_e n), n - 1) moves to R_I + sigma eps, I the first nucleus whose cumulative charge exceeds
    u_n sum Z.  Returns (r', log(q(r_old) / q(r_new))) with q(x) = sum_J Z_J exp(-|x - R_J|^2 / (2 sigma^2))."""
    n = r.shape[0]
    e = min(int(d[0] * n), n - 1)
    cz = np.cumsum(np.asarray(Z, np.float64))
    hit = np.nonzero(cz > d[1] * cz[-1])[0]
    I = int(hit[0]) if len(hit) else len(Z) - 1
    rn = r.copy()
    rn[e] = np.asarray(R, np.float64)[I] + sigma * np.asarray(d[2:5], np.float64)

    def q(x):
        return np.sum(np.asarray(Z, np.float64) * np.exp(-0.5 / sigma**2 * np.sum((x - np.asarray(R, np.float64)) ** 2, axis=-1)))

    return rn, np.log(q(r[e])) - np.log(q(rn[e]))


def mcmc_jump_block(prob, p, r, draws, log_u, sigma):
    """Metropolis block of jumps to the nuclei (``mcmc_steps_low_rank`` with ``proposal_jump_to_atom``,
    ``mcmc.py:164-193, 196-275``) with externally supplied draws [steps, 5]: accept iff
    log_ratio_proposal + 2 (log|psi'| - log|psi|) > log_u[s].  Returns (r, log_prob, n_accept, margins)."""
    lp = 2.0 * logpsi(prob, p, r)[1]
    n_acc = 0
    margins = []
    for s in range(draws.shape[0]):
        rn, plr = jump_proposal(prob.R, prob.Z, r, draws[s], sigma)
        lpn = 2.0 * logpsi(prob, p, rn)[1]
        m = plr + (lpn - lp) - log_u[s]
        margins.append(m)
        if m > 0:
            r, lp = rn, lpn
            n_acc += 1
    return r, lp, n_acc, np.array(margins)



def closest_k(dist, dist_max, k):
    """``_get_closest_k`` (``mcmc.py:114-117``): the k smallest distances (stable: lower index first on ties, as
    ``jax.lax.top_k`` of -dist), NO_NEIGHBOUR where the distance exceeds dist_max."""
    order = np.argsort(dist, kind="stable")[:k]
    return np.where(dist[order] <= dist_max, order, NO_NEIGHBOUR)


def cluster_proposal(r, d, k, radius, width, center):
    """``proposal_cluster_update`` (``mcmc.py:119-161``) for draws d = (u_center, eps [5][k][3]) and a given center:
    the k closest electrons within radius move by width * eps[t] (row i to the i-th closest); the first of 5 draws
    whose moved center has the same closest set is proposed with log ratio 0, else the first draw with -inf.
    Returns (r', log ratio)."""
    idx = closest_k(np.linalg.norm(r - r[center], axis=-1), radius, k)
    eps = np.asarray(d[1:], np.float64).reshape(5, k, 3)
    props, valid = [], []
    for t in range(5):
        rp = r.copy()
        for i in range(k):
            if idx[i] != NO_NEIGHBOUR:
                rp[idx[i]] = rp[idx[i]] + eps[t, i] * width
        rev = closest_k(np.linalg.norm(rp - rp[center], axis=-1), radius, k)
        props.append(rp)
        valid.append(float(np.all(np.sort(idx) == np.sort(rev))))
    t = int(np.argmax(valid))
    return props[t], (0.0 if valid[t] > 0 else -np.inf)


def mcmc_cluster_block(prob, p, r, draws, log_u, width, k, radius, random_sweep=False, offset=0):
    """Metropolis block of cluster updates (``mcmc_steps_low_rank`` with ``proposal_cluster_update``) with
    externally supplied draws [steps, 1 + 15 k]: center (offset + s) mod n, or min(floor(u_center n), n - 1) for a
    random sweep.  Returns (r, log_prob, n_accept, margins)."""
    n = r.shape[0]
    lp = 2.0 * logpsi(prob, p, r)[1]
    n_acc = 0
    margins = []
    for s in range(draws.shape[0]):
        center = min(int(draws[s][0] * n), n - 1) if random_sweep else (offset + s) % n
        rn, plr = cluster_proposal(r, draws[s], k, radius, width, center)
        lpn = 2.0 * logpsi(prob, p, rn)[1]
        m = plr + (lpn - lp) - log_u[s]
        margins.append(m)
        if m > 0:
            r, lp = rn, lpn
            n_acc += 1
    return r, lp, n_acc, np.array(margins)


def mcmc_single_block(prob, p, r, noise, log_u, width, offset=0):
    """Single-electron Metropolis block: ``proposal_single_electron`` (``mcmc.py:100-111``) driven by
    ``mcmc_steps_low_rank`` (``mcmc.py:196-275``) with externally supplied draws.  Step s moves electron
    (offset + s) mod n by width * noise[s] ([steps, 3]); accept iff 2 (log|psi'| - log|psi|) > log_u[s].  log|psi'|
    is evaluated in full (the reference's low-rank update reaches the same value, ``tests/test_low_rank.py``).
    Returns (r, log_prob, n_accept, margins)."""
    n = r.shape[0]
    lp = 2.0 * logpsi(prob, p, r)[1]
    n_acc = 0
    margins = []
    for s in range(noise.shape[0]):
        e = (offset + s) % n
        rn = r.copy()
        rn[e] = r[e] + noise[s] * width
        lpn = 2.0 * logpsi(prob, p, rn)[1]
        m = (lpn - lp) - log_u[s]
        margins.append(m)
        if m > 0:
            r, lp = rn, lpn
            n_acc += 1
    return r, lp, n_acc, np.array(margins)


def mcmc_low_rank_block(prob, p, r, propose, log_u):
    """``mcmc_steps_low_rank`` (``mcmc.py:196-275``) for one walker with the state carried between steps:
    ``propose(s, r)`` returns (r', moved electrons, proposal log ratio); log|psi'| comes from
    ``logpsi_low_rank_update`` and the state of an accepted proposal replaces the current one.  Returns
    (r, log_prob, n_accept, margins, changed_max) with changed_max the elementwise maximum over the steps of the
    proposals' ``changed_counts`` (the move statics the reference accumulates, ``mcmc.py:231-235``)."""
    (_, l), st = logpsi_with_state(prob, p, r)
    lp = 2.0 * l
    n_acc = 0
    margins = []
    cmax = np.zeros(3, np.int64)
    for s in range(len(log_u)):
        rn, idx, plr = propose(s, r)
        cmax = np.maximum(cmax, changed_counts(prob, r, rn, idx))
        (_, ln), stn = logpsi_low_rank_update(prob, p, rn, idx, st)
        m = plr + (2.0 * ln - lp) - log_u[s]
        margins.append(m)
        if m > 0:
            r, lp, st = rn, 2.0 * ln, stn
            n_acc += 1
    return r, lp, n_acc, np.array(margins), cmax


def single_electron_low_rank_block(prob, p, r, noise, log_u, width, offset=0):
    """``mcmc_single_block``'s moves through ``mcmc_low_rank_block``."""
    n = r.shape[0]

    def propose(s, r):
        e = (offset + s) % n
        rn = r.copy()
        rn[e] = r[e] + noise[s] * width
        return rn, np.array([e]), 0.0

    return mcmc_low_rank_block(prob, p, r, propose, log_u)


def cluster_low_rank_block(prob, p, r, draws, log_u, width, k, radius, random_sweep=False, offset=0):
    """``mcmc_cluster_block``'s moves through ``mcmc_low_rank_block``; the moved electrons are the center's k closest
    before the move, NO_NEIGHBOUR-padded (``proposal_cluster_update``, ``mcmc.py:141-143``)."""
    n = r.shape[0]

    def propose(s, r):
        center = min(int(draws[s][0] * n), n - 1) if random_sweep else (offset + s) % n
        idx = closest_k(np.linalg.norm(r - r[center], axis=-1), radius, k)
        rn, plr = cluster_proposal(r, draws[s], k, radius, width, center)
        return rn, idx, plr

    return mcmc_low_rank_block(prob, p, r, propose, log_u)


# =============================================================================== Philox draws of the device blocks
# The device Metropolis blocks draw from Philox4x32-10 (Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as
# easy as 1, 2, 3", SC'11): 10 rounds of the multiply-xor round function with the Weyl key schedule.  This numpy
# restatement regenerates the all-electron block's draws on the CPU, so that the CPU baseline can run the same
# Metropolis block as the device (the reference itself draws from jax's threefry, which cannot be reproduced here).
PHILOX_M = (0xD2511F53, 0xCD9E8D57)
PHILOX_W = (0x9E3779B9, 0xBB67AE85)
_U32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(ctr, key):
    """Philox4x32-10 of counters ctr [..., 4] under keys key [..., 2] (uint32 values): [..., 4] uint32."""
    ctr = np.asarray(ctr, np.uint64)
    key = np.asarray(key, np.uint64)
    c0, c1, c2, c3 = (ctr[..., i] for i in range(4))
    k0, k1 = key[..., 0], key[..., 1]
    m0, m1 = np.uint64(PHILOX_M[0]), np.uint64(PHILOX_M[1])
    for _ in range(10):
        p0, p1 = m0 * c0, m1 * c2  # 32 x 32 -> 64-bit products, exact in uint64
        c0, c1, c2, c3 = (p1 >> np.uint64(32)) ^ c1 ^ k0, p1 & _U32, (p0 >> np.uint64(32)) ^ c3 ^ k1, p0 & _U32
        k0 = (k0 + np.uint64(PHILOX_W[0])) & _U32
        k1 = (k1 + np.uint64(PHILOX_W[1])) & _U32
    return np.stack([c0, c1, c2, c3], -1).astype(np.uint32)


def _philox_key(seed, counter):
    k = (int(seed) ^ ((int(counter) >> 32) * 0x9E3779B97F4A7C15)) & 0xFFFFFFFFFFFFFFFF
    return np.array([k & 0xFFFFFFFF, k >> 32], np.uint64)


def _u01(x):
    return ((np.asarray(x, np.uint64) >> np.uint64(8)).astype(np.float64) + 0.5) * (1.0 / 16777216.0)


def philox_all_electron_noise(seed, counter, step, walker, n):
    """The device's all-electron proposal normals eps [n, 3] (float32) of one walker and step: counter (step,
    walker, electron, counter), Box-Muller on the four uniforms."""
    ctr = np.zeros((n, 4), np.uint64)
    ctr[:, 0], ctr[:, 1], ctr[:, 2], ctr[:, 3] = step, walker, np.arange(n), int(counter) & 0xFFFFFFFF
    x = philox4x32_10(ctr, np.broadcast_to(_philox_key(seed, counter), (n, 2)))
    r1, t1 = np.sqrt(-2.0 * np.log(_u01(x[:, 0]))), 2.0 * np.pi * _u01(x[:, 1])
    r2, t2 = np.sqrt(-2.0 * np.log(_u01(x[:, 2]))), 2.0 * np.pi * _u01(x[:, 3])
    return np.stack([r1 * np.cos(t1), r1 * np.sin(t1), r2 * np.cos(t2)], -1).astype(np.float32)


def philox_log_u(seed, counter, step, walker):
    """The device's Metropolis log-uniform of one walker and step: counter (step, walker, 0xFFFFFFFF, counter)."""
    ctr = np.array([[step, walker, 0xFFFFFFFF, int(counter) & 0xFFFFFFFF]], np.uint64)
    return float(np.log(_u01(philox4x32_10(ctr, _philox_key(seed, counter)[None])[0, 0])))


def mcmc_block_philox(prob, p, r, steps, width, seed, counter, walker):
    """The all-electron Metropolis block (``mcmc.py:38-97``) of walker index ``walker`` with the device's Philox
    draws: positions stay float32 (r' = r + width eps, one rounding), log|psi| in FP64.  Returns (r float32,
    n_accept, margins)."""
    r = np.asarray(r, np.float32)
    w32 = np.float32(width)
    lp = 2.0 * logpsi(prob, p, r.astype(np.float64))[1]
    n_acc, margins = 0, []
    for s in range(steps):
        eps = philox_all_electron_noise(seed, counter, s, walker, r.shape[0])
        rn = (r.astype(np.float64) + np.float64(w32) * eps.astype(np.float64)).astype(np.float32)
        lpn = 2.0 * logpsi(prob, p, rn.astype(np.float64))[1]
        m = (lpn - lp) - philox_log_u(seed, counter, s, walker)
        margins.append(m)
        if m > 0:
            r, lp = rn, lpn
            n_acc += 1
    return r, n_acc, np.array(margins)
