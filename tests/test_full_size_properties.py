"""Parity at the full 1M x 784 config-2 size, through properties that need no
full CPU fit.

From the engine's own top-k / top-m lists, the neighbourhood of a sampled
point p is rebuilt exactly as the reference defines it
(src/sDbscan.cpp:243-296, :374-400): p's candidates through its 2k lists plus
every point that meets p through one of its lists, within eps, p excluded,
duplicates once.  Distances are screened in float64; a pair within 1e-5 of
eps is decided with the oracle's FP32 transform and distance (the engine's
numerical contract).  Checked for the sample:
  - the engine's neighbourhood size (degree) and core flag;
  - labels: a core point shares its label with every core neighbour; a
    non-core point carries the smallest label among its core neighbours, or
    -1 (src/sDbscan.cpp:509-637; cluster ids grow with the smallest core index).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, DIM, D, K, M, EPS, MINPTS = 1_000_000, 784, 1024, 10, 50, 0.25, 50


def _decide(port, xp_raw, rows_raw, d64):
    """Exact FP32 eps decision for the pairs whose float64 distance is within
    1e-5 of eps; the float64 decision elsewhere."""
    out = d64 <= EPS
    near = np.nonzero(np.abs(d64 - EPS) <= 1e-5)[0]
    if near.size:
        xt, rc = port.transform(xp_raw[None, :], "Cosine")
        assert rc == 0
        yt, rc = port.transform(rows_raw[near], "Cosine")
        assert rc == 0
        for t, j in enumerate(near):
            out[j] = port.distance(xt[0], yt[t], "Cosine") <= EPS
    return out


def test_full_size_degrees_and_labels(port):
    import torch
    from sdbscan_gb300 import capi, datasets
    X, _ = datasets.cfg2_mnist_like_torch(N, DIM, seed=2007, device="cuda")
    torch.cuda.synchronize()
    eng = capi.Engine(N, DIM)
    eng.set_params(n_proj=D, topK=K, topM=M, distance="Cosine", random_seed=42)
    eng.fit_sdbscan_device(X.data_ptr(), EPS, MINPTS)
    labels, ncl = eng.labels()
    core, deg = eng.core()
    topK = eng.topk().astype(np.int64)
    topM = eng.topm()
    eng.close()

    # list ids of each point's slots, the candidates of each list, and the
    # inverted indexes (list -> member points, point -> lists holding it)
    lists = topK + np.where(np.arange(2 * K) >= K, D, 0)[None, :]
    cand = np.concatenate([topM[:, :M], topM[:, M:]], axis=0)  # list l = side * D + r
    flat = lists.ravel()
    order = np.argsort(flat, kind="stable")
    mem_pts = order // (2 * K)
    mem_off = np.searchsorted(flat[order], np.arange(2 * D + 1))
    cflat = cand.ravel()
    corder = np.argsort(cflat, kind="stable")
    hub_lists = corder // M
    hub_off = np.searchsorted(cflat[corder], np.arange(N + 1))

    rng = np.random.default_rng(11)
    nhub = hub_off[1:] - hub_off[:-1]
    non_hubs = rng.choice(np.nonzero(nhub == 0)[0], 40, replace=False)
    hubs = [p for p in rng.permutation(np.nonzero(nhub > 0)[0])
            if sum(mem_off[l + 1] - mem_off[l] for l in hub_lists[hub_off[p]:hub_off[p + 1]]) <= 20000][:10]
    sample = list(non_hubs) + hubs
    assert len(hubs) >= 5

    Xn = X / torch.linalg.vector_norm(X.double(), dim=1, keepdim=True).float()
    checked_core = checked_border = 0
    for p in sample:
        fwd = cand[lists[p]].ravel()
        rev = np.concatenate([mem_pts[mem_off[l]:mem_off[l + 1]] for l in hub_lists[hub_off[p]:hub_off[p + 1]]]
                             + [np.empty(0, np.int64)])
        nb = np.unique(np.concatenate([fwd, rev]).astype(np.int64))
        nb = nb[nb != p]
        idx = torch.from_numpy(nb).cuda()
        d64 = (1.0 - (Xn[idx].double() @ Xn[p].double())).cpu().numpy()
        within = _decide(port, X[p].cpu().numpy(), X[idx].cpu().numpy(), d64)
        neigh = nb[within]
        assert deg[p] == neigh.size, (p, deg[p], neigh.size)
        assert core[p] == (neigh.size >= MINPTS - 1)
        core_nb = neigh[core[neigh] == 1]
        if core[p]:
            assert labels[p] >= 0 and np.all(labels[core_nb] == labels[p])
            checked_core += 1
        else:
            want = labels[core_nb].min() if core_nb.size else -1
            assert labels[p] == want, (p, labels[p], want)
            checked_border += 1
    assert ncl == (labels.max() + 2 if labels.max() >= 0 else 2)
    assert checked_core > 0
