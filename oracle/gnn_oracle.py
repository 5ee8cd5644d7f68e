"""CPU restatement of the learned-start network (TEST INFRASTRUCTURE ONLY).

The checker for the GPU library's mesh-graph network: forward pass, loss and the gradient with
respect to every parameter, in float64 numpy.  With ``bf16=True`` the operands of each matrix
product are rounded to BF16 (round to nearest even) at the same points as the GPU's tensor-core
kernels, so the two differ only by accumulation order (FP32 on the GPU, FP64 here).  With
``bf16=False`` it is the exact network, which the finite-difference test pins.

Parameter vector layout (float32 in the library): We [64x16], be [64], then per layer
W1 [64x128], b1 [64], W2 [64x64], b2 [64] (4 layers), then Wd [3x64], bd [3] (outputs: u, v and
the log-viscosity).
"""
from __future__ import annotations

import numpy as np

C, FIN, LAYERS, NB, OUT = 64, 16, 4, 3, 3


def layout():
    off, o = {}, 0

    def add(name, shape):
        nonlocal o
        off[name] = (o, shape)
        o += int(np.prod(shape))

    add("We", (C, FIN))
    add("be", (C,))
    for l in range(LAYERS):
        add(f"W1_{l}", (C, 2 * C))
        add(f"b1_{l}", (C,))
        add(f"W2_{l}", (C, C))
        add(f"b2_{l}", (C,))
    add("Wd", (OUT, C))
    add("bd", (OUT,))
    return off, o


OFFSETS, NPARAMS = layout()


def unpack(p):
    return {k: np.asarray(p[o:o + int(np.prod(s))], dtype=np.float64).reshape(s) for k, (o, s) in OFFSETS.items()}


def pack(d):
    p = np.zeros(NPARAMS, np.float64)
    for k, (o, s) in OFFSETS.items():
        p[o:o + int(np.prod(s))] = np.asarray(d[k]).reshape(-1)
    return p


def bf16(a):
    """Round to BF16 (nearest even) and back, through float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + 0x7FFF
    return (((u + r) >> 16) << 16).view(np.float32).astype(np.float64)


def _mean_nbr(nbr, h):
    n = h.shape[0]
    a = np.zeros_like(h)
    deg = np.zeros(n)
    for q in range(NB):
        j = nbr[:, q]
        ok = j >= 0
        a[ok] += h[j[ok]]
        deg += ok
    inv = np.where(deg > 0, 1.0 / np.maximum(deg, 1), 0.0)
    return a * inv[:, None], inv


def forward(p, nbr, x, bf=True):
    P = unpack(p)
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    x = np.asarray(x, dtype=np.float64)
    cache = {"x": x}
    h = np.maximum(r(x) @ r(P["We"]).T + P["be"], 0.0)
    cache["h0"] = h
    hs, ts, zs = [h], [], []
    for l in range(LAYERS):
        a, inv = _mean_nbr(nbr, h)
        z = np.concatenate([r(h), r(a)], axis=1)
        t = r(np.maximum(z @ r(P[f"W1_{l}"]).T + P[f"b1_{l}"], 0.0))
        h = h + (t @ r(P[f"W2_{l}"]).T + P[f"b2_{l}"])
        zs.append(z)
        ts.append(t)
        hs.append(h)
        cache["inv"] = inv
    y = h @ P["Wd"].T + P["bd"]
    cache.update(hs=hs, ts=ts, zs=zs)
    return y, cache


def loss_grad(p, nbr, x, target, w, bf=True):
    """(loss, grad) with loss = sum_i w_i |y_i - target_i|^2."""
    P = unpack(p)
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    y, c = forward(p, nbr, x, bf)
    e = y - target
    loss = float(np.sum(w * np.sum(e * e, axis=1)))
    G = {k: np.zeros(s) for k, (o, s) in OFFSETS.items()}
    dy = 2.0 * w[:, None] * e
    hL = c["hs"][-1]
    G["Wd"] = dy.T @ hL
    G["bd"] = dy.sum(axis=0)
    dh = dy @ P["Wd"]
    inv = c["inv"]
    for l in reversed(range(LAYERS)):
        t, z = c["ts"][l], c["zs"][l]
        dt = r(dh) @ r(P[f"W2_{l}"])
        ds = dt * (t > 0)
        dz = r(ds) @ r(P[f"W1_{l}"])
        G[f"W2_{l}"] = r(dh).T @ t
        G[f"b2_{l}"] = dh.sum(axis=0)
        G[f"W1_{l}"] = r(ds).T @ z
        G[f"b1_{l}"] = ds.sum(axis=0)
        dacc = dh + dz[:, :C]
        dA = dz[:, C:] * inv[:, None]
        dh_in = dacc.copy()
        for q in range(NB):
            i = nbr[:, q]
            ok = i >= 0
            dh_in[ok] += dA[i[ok]]
        dh = dh_in
    ds_e = dh * (c["h0"] > 0)
    G["We"] = r(ds_e).T @ r(c["x"])
    G["be"] = ds_e.sum(axis=0)
    return loss, pack(G)


def random_graph(n, seed=0):
    """A random symmetric graph with at most 3 neighbours per node (a perturbed ring lattice)."""
    rng = np.random.default_rng(seed)
    nbr = -np.ones((n, NB), np.int32)
    deg = np.zeros(n, int)
    perm = rng.permutation(n)
    for k in range(n):                      # ring edges
        i, j = perm[k], perm[(k + 1) % n]
        if deg[i] < NB and deg[j] < NB and i != j and j not in nbr[i]:
            nbr[i, deg[i]] = j
            nbr[j, deg[j]] = i
            deg[i] += 1
            deg[j] += 1
    for _ in range(n // 2):                 # chords
        i, j = rng.integers(0, n, 2)
        if i != j and deg[i] < NB and deg[j] < NB and j not in nbr[i]:
            nbr[i, deg[i]] = j
            nbr[j, deg[j]] = i
            deg[i] += 1
            deg[j] += 1
    return nbr
