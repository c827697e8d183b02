"""Differentiable personalised PageRank (eeg_ppr_*) on the GPU.

Parity: forward X, adjoint L and the three gradients against the FP64 oracle (oracle.ppr); central
finite differences (eps = 1e-3) through a torch.autograd.Function wrapper (test harness only); the
single-column loop with accumulation against the batched rows; hubs spanning several chunk groups;
size-independent identities at larger sizes (duality c^T x = (1-d) t^T lambda, row-scale invariance
sum_v w_uv dL/dw_uv = 0); determinism; error statuses.

Tolerances: X and L within 1e-6 normalised L1 per column of the FP64 solution (the FP32 solve stops at
tol 1e-7 on its own residual bound); edge gradients within 1e-5 normalised L1.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

D = 0.85


def _graph(E, scale, ef, seed, K=8, extra=None):
    n = 1 << scale
    s, d, _ = E.gen_rmat(scale, ef, seed=seed, wmin=1, wmax=63)
    s, d = np.asarray(s, np.uint32), np.asarray(d, np.uint32)
    if extra is not None:
        s = np.concatenate([s, extra[0]]).astype(np.uint32)
        d = np.concatenate([d, extra[1]]).astype(np.uint32)
    rng = np.random.default_rng(seed + 100)
    w = (1.0 - rng.random(s.size)).astype(np.float32)  # U(0, 1]
    vg = E.VirtualGraph.build(n, s, d, None, K=K, reverse=True, edge_ids=True)
    return n, s, d, w, vg


def _teleport(n, C, seeds_per_col, rng):
    T = np.zeros((n, C), np.float32)
    for k in range(C):
        T[rng.choice(n, seeds_per_col, replace=False), k] = 1.0 / seeds_per_col
    return T


def _nl1(a, b):
    """normalised L1 per column (max over columns)"""
    a = np.asarray(a, np.float64).reshape(a.shape[0], -1)
    b = np.asarray(b, np.float64).reshape(b.shape[0], -1)
    return float((np.abs(a - b).sum(0) / np.maximum(np.abs(b).sum(0), 1e-300)).max())


def _rel_l1(a, b):
    a, b = np.asarray(a, np.float64).ravel(), np.asarray(b, np.float64).ravel()
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))


@pytest.mark.parametrize("K", [4, 8, 16])
@pytest.mark.parametrize("C", [1, 5, 32, 33, 64])  # plain form; 128-B rows (<= 32 columns); 256-B rows
def test_ppr_matches_fp64_oracle(gpu, K, C):
    E = gpu
    n, s, d, w, vg = _graph(E, 11, 16, seed=K + C, K=K)
    rng = np.random.default_rng(C)
    T = _teleport(n, C, 32, rng)
    G = rng.standard_normal((n, C)).astype(np.float32)
    ref = oracle.ppr(n, s, d, w.astype(np.float64), T, G, damping=D)
    with E.PPR(vg, C) as p:
        p.set_weights(w)
        X, rf = p.forward(T)
        assert rf["iterations"] > 10
        out, ra = p.adjoint(G)
    assert _nl1(X, ref["X"]) <= 1e-6, _nl1(X, ref["X"])
    # the adjoint values are checked through dT = (1-d) L
    assert _nl1(out["dt"], ref["gT"]) <= 1e-6, _nl1(out["dt"], ref["gT"])
    assert _rel_l1(out["dwn"], ref["gWn"]) <= 1e-5, _rel_l1(out["dwn"], ref["gWn"])
    assert _rel_l1(out["dw"], ref["gw"]) <= 1e-5, _rel_l1(out["dw"], ref["gw"])
    vg.close()


def test_ppr_hubs_span_groups(gpu):
    """A vertex with 12000 in- and out-edges: 12000/128 chunks -> 3 groups of 32 per direction."""
    E = gpu
    hub_n = 12000
    nb = np.arange(1, hub_n + 1, dtype=np.uint32) % (1 << 14)
    extra = (np.concatenate([nb, np.zeros(hub_n, np.uint32)]), np.concatenate([np.zeros(hub_n, np.uint32), nb]))
    for K in (4, 8, 16):
        n, s, d, w, vg = _graph(E, 14, 4, seed=3, K=K, extra=extra)
        rng = np.random.default_rng(K)
        for C in (1, 20, 64):
            T = _teleport(n, C, 32, rng)
            T[0, :] += 0.5
            G = rng.standard_normal((n, C)).astype(np.float32)
            ref = oracle.ppr(n, s, d, w.astype(np.float64), T, G, damping=D)
            with E.PPR(vg, C) as p:
                p.set_weights(w)
                X, _ = p.forward(T)
                out, _ = p.adjoint(G)
            assert _nl1(X, ref["X"]) <= 1e-6, (K, C, _nl1(X, ref["X"]))
            assert _nl1(out["dt"], ref["gT"]) <= 1e-6, (K, C)
            assert _rel_l1(out["dw"], ref["gw"]) <= 1e-5, (K, C, _rel_l1(out["dw"], ref["gw"]))
        vg.close()


def test_ppr_loop_of_columns_equals_batch(gpu):
    """The plain form looped over the columns with accumulation gives the batched gradients."""
    E = gpu
    n, s, d, w, vg = _graph(E, 12, 16, seed=5)
    rng = np.random.default_rng(5)
    C = 8
    T = _teleport(n, C, 32, rng)
    G = rng.standard_normal((n, C)).astype(np.float32)
    with E.PPR(vg, C) as pb:
        pb.set_weights(w)
        Xb, _ = pb.forward(T)
        ob, _ = pb.adjoint(G)
    with E.PPR(vg, 1) as p1:
        p1.set_weights(w)
        Xs, dts = [], []
        for k in range(C):
            x, _ = p1.forward(np.ascontiguousarray(T[:, k:k + 1]))
            o, _ = p1.adjoint(np.ascontiguousarray(G[:, k:k + 1]), accumulate=k > 0,
                              outputs=("dw", "dwn", "dt") if k == C - 1 else ("dt",))
            Xs.append(x[:, 0])
            dts.append(o["dt"][:, 0])
    assert _nl1(np.stack(Xs, 1), Xb) <= 2e-6
    assert _nl1(np.stack(dts, 1), ob["dt"]) <= 2e-6
    assert _rel_l1(o["dw"], ob["dw"]) <= 2e-5
    assert _rel_l1(o["dwn"], ob["dwn"]) <= 2e-5
    vg.close()


class _PPRFunction:
    """torch.autograd.Function over the C ABI (test harness only): (w, T) -> X."""

    @staticmethod
    def make(torch, ppr):
        class F(torch.autograd.Function):
            @staticmethod
            def forward(ctx, w, T):
                ppr.set_weights(w.data_ptr())
                X = torch.empty_like(T)
                ppr.forward(T.data_ptr(), X.data_ptr())
                return X

            @staticmethod
            def backward(ctx, gX):
                gX = gX.contiguous()
                dw = torch.empty(ppr.m, dtype=torch.float32, device=gX.device)
                dT = torch.empty_like(gX)
                ppr.adjoint(gX.data_ptr(), out_ptrs={"dw": dw.data_ptr(), "dt": dT.data_ptr()})
                return dw, dT

        return F


def test_ppr_autograd_finite_differences(gpu):
    torch = pytest.importorskip("torch")
    E = gpu
    n, s, d, w, vg = _graph(E, 9, 8, seed=11)
    rng = np.random.default_rng(11)
    C = 4
    T = _teleport(n, C, 16, rng)
    Cg = rng.standard_normal((n, C)).astype(np.float32)
    with E.PPR(vg, C) as p:
        F = _PPRFunction.make(torch, p)
        wt = torch.tensor(w, device="cuda", requires_grad=True)
        Tt = torch.tensor(T, device="cuda", requires_grad=True)
        ct = torch.tensor(Cg, device="cuda")
        loss = (F.apply(wt, Tt) * ct).sum()
        loss.backward()
        gw, gT = wt.grad.cpu().numpy(), Tt.grad.cpu().numpy()

        def L(wv, Tv):
            with torch.no_grad():
                return float((F.apply(torch.tensor(wv, device="cuda"), torch.tensor(Tv, device="cuda")) * ct)
                             .double().sum())

        eps = 1e-3
        scale_w = np.abs(gw).max()
        for e in rng.choice(s.size, 12, replace=False):
            wp, wm = w.copy(), w.copy()
            wp[e] += eps
            wm[e] -= eps
            fd = (L(wp, T) - L(wm, T)) / (2 * eps)
            assert abs(fd - gw[e]) <= 2e-3 * scale_w + 1e-3 * abs(gw[e]), (e, fd, gw[e])
        scale_t = np.abs(gT).max()
        for _ in range(8):
            i, k = int(rng.integers(0, n)), int(rng.integers(0, C))
            Tp, Tm = T.copy(), T.copy()
            Tp[i, k] += eps
            Tm[i, k] -= eps
            fd = (L(w, Tp) - L(w, Tm)) / (2 * eps)
            assert abs(fd - gT[i, k]) <= 2e-3 * scale_t + 1e-3 * abs(gT[i, k]), (i, k, fd, gT[i, k])
    # and the same gradients from the FP64 oracle
    ref = oracle.ppr(n, s, d, w.astype(np.float64), T, Cg, damping=D)
    assert _rel_l1(gw, ref["gw"]) <= 1e-5
    assert _nl1(gT, ref["gT"]) <= 1e-6
    vg.close()


def test_ppr_identities_at_scale(gpu):
    """R-MAT s18 (4.2M edges) x 64 columns: duality and row-scale invariance (size-independent checks)."""
    torch = pytest.importorskip("torch")
    E = gpu
    n, s, d, w, vg = _graph(E, 18, 16, seed=1)
    rng = np.random.default_rng(1)
    T = _teleport(n, 64, 32, rng)
    G = rng.standard_normal((n, 64)).astype(np.float32)
    Tt, Gt = torch.tensor(T, device="cuda"), torch.tensor(G, device="cuda")
    X = torch.empty_like(Tt)
    dT = torch.empty_like(Tt)
    dw = torch.empty(s.size, dtype=torch.float32, device="cuda")
    with E.PPR(vg, 64) as p:
        p.set_weights(w)
        _, rf = p.forward(Tt.data_ptr(), X.data_ptr())
        _, ra = p.adjoint(Gt.data_ptr(), out_ptrs={"dw": dw.data_ptr(), "dt": dT.data_ptr()})
        X2 = torch.empty_like(Tt)
        p.forward(Tt.data_ptr(), X2.data_ptr())
        assert torch.equal(X, X2)  # deterministic
    lhs = float((Gt.double() * X.double()).sum())
    rhs = float((Tt.double() * dT.double()).sum())  # dT = (1-d) L
    assert abs(lhs - rhs) <= 1e-5 * (Gt.double().abs() * X.double().abs()).sum().item()
    # sum_v w_uv dL/dw_uv = 0 per source u
    src = torch.tensor(s.astype(np.int64), device="cuda")
    wt = torch.tensor(w, device="cuda").double()
    tot = torch.zeros(n, dtype=torch.float64, device="cuda").index_add_(0, src, wt * dw.double())
    mag = torch.zeros(n, dtype=torch.float64, device="cuda").index_add_(0, src, (wt * dw.double()).abs())
    assert float((tot.abs() - 1e-4 * mag).max()) <= 1e-12
    assert rf["iterations"] > 20 and ra["iterations"] > 20
    vg.close()


def test_ppr_errors(gpu):
    E = gpu
    n = 64
    s = np.arange(n, dtype=np.uint32)
    d = (s + 1) % n
    vg_plain = E.VirtualGraph.build(n, s, d, None, K=8, reverse=True)
    with pytest.raises(E.EEGError):
        E.PPR(vg_plain, 4)
    vg_plain.close()
    vg = E.VirtualGraph.build(n, s, d, None, K=8, reverse=True, edge_ids=True)
    with pytest.raises(E.EEGError):
        E.PPR(vg, 65)
    with E.PPR(vg, 2) as p:
        T = np.zeros((n, 2), np.float32)
        T[0] = 1
        with pytest.raises(E.EEGError):
            p.forward(T)  # no weights yet
        with pytest.raises(E.EEGError):
            p.set_weights(-np.ones(n, np.float32))
        p.set_weights(np.ones(n, np.float32))
        with pytest.raises(E.EEGError):
            p.adjoint(T)  # no forward yet
        X, _ = p.forward(T)
        # a directed ring: x_{i+1} = d x_i, x_0 = (1-d) + d x_{n-1}
        ref = oracle.ppr_solve(n, s, d, np.ones(n), T, damping=D)[0]
        assert _nl1(X, ref) <= 1e-6
    vg.close()


def test_ppr_column_shards_sum_to_batch(gpu):
    """Column sharding (one shard per GPU): each shard is an independent solve over its columns, and the
    edge gradients of the whole batch are the sum of the shards' (the loss is a sum over columns)."""
    E = gpu
    n, s, d, w, vg = _graph(E, 12, 16, seed=21, K=8)
    rng = np.random.default_rng(21)
    C = 64
    T = _teleport(n, C, 32, rng)
    G = rng.standard_normal((n, C)).astype(np.float32)
    with E.PPR(vg, C) as p:
        p.set_weights(w)
        X, _ = p.forward(T)
        full, _ = p.adjoint(G)
    for world in (2, 3):
        cols = E.shard_columns(C, world)
        assert sorted(c for sh in cols for c in sh) == list(range(C))
        dw = np.zeros_like(full["dw"], dtype=np.float64)
        for sh in cols:
            with E.PPR(vg, len(sh)) as p:
                p.set_weights(w)
                Xs, _ = p.forward(np.ascontiguousarray(T[:, sh]))
                out, _ = p.adjoint(np.ascontiguousarray(G[:, sh]))
            assert _nl1(Xs, X[:, sh]) <= 2e-6
            assert _nl1(out["dt"], full["dt"][:, sh]) <= 2e-6
            dw += out["dw"]
        assert _rel_l1(dw, full["dw"]) <= 1e-5, (world, _rel_l1(dw, full["dw"]))
    vg.close()
