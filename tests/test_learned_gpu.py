"""Learned preconditioner: the device network against a PyTorch-CPU restatement
(forward, loss and parameter gradients), training on solver-generated pairs, the
learned flexible CG against Jacobi, and the versioned parameter file."""
import numpy as np
import pytest

from helpers import make_problem

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import torch.nn.functional as F  # noqa: E402

C8, TAPS = 8, 27


def build(be, pb):
    import gridap_gb300 as G
    ranks = be.distribute(range(int(np.prod(pb.np))))
    model = G.CartesianDiscreteModel(ranks, pb.np, pb.domain, pb.n)
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, float, 1), dirichlet_tags="boundary")
    U = G.TrialFESpace(0.0, V)
    dO = G.Measure(G.Triangulation(model), 2)
    f = pb.f_nodal if pb.f_nodal is not None else pb.f_const
    op = G.AffineFEOperator(G.integral_grad_grad(pb.kappa, dO), G.integral_source(f, dO), U, V)
    return model, V, op


def gid_to_node(V):
    n = V.num_free_dofs()
    out = np.zeros(n, dtype=np.int64)
    for p in range(V.model.num_parts):
        li = V.gids.partition()[p]
        nodes = V.dof_nodes(p)
        own = li.local_to_owner == p
        out[li.local_to_global[own]] = nodes[own]
    return out


def global_matrix(op):
    import scipy.sparse as sps
    n = op.matrix.n_global
    rows, cols, vals = [], [], []
    for p, (rp, ci, vv) in enumerate(op.matrix.csr_parts()):
        rpart, cpart = op.matrix.row_partition[p], op.matrix.col_partition[p]
        nown = rpart.own_length()
        colg = cpart.local_to_global
        for r in range(nown):
            s, e = rp[r], rp[r + 1]
            rows.append(np.full(e - s, rpart.own_to_global[r]))
            cols.append(colg[ci[s:e]])
            vals.append(vv[s:e])
    return sps.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def torch_net(params, kappa_cells, cells, r_gid, node_of_gid, dinv, levels, coarse_start=False):
    """The same network in float64 PyTorch on the CPU; returns z (gid order).

    S^T S x is taken as the gradient of 0.5 |S x|^2 (autograd), an independent route to
    the decoder that the device computes as the explicit adjoint of the encoder; with
    coarse_start the restriction R sits inside the autograd graph, so R^T is its exact
    adjoint (the device uses P / 8)."""
    N = [c + 1 for c in cells]
    nlat = int(np.prod(N))
    off = 0

    def take(count, shape):
        nonlocal off
        t = params[off:off + count].reshape(shape)
        off += count
        return t
    W = [take(C8 * (1 if l == 0 else C8) * TAPS, (C8, 1 if l == 0 else C8, 3, 3, 3)) for l in range(levels)]
    G = [take(C8 * TAPS, (C8, 1, 3, 3, 3)) for _ in range(levels)]
    Bs = [take(C8, (C8,)) for _ in range(levels)]
    assert off == params.numel()
    # node feature: log mean kappa of the cells around each node
    kc = torch.tensor(kappa_cells, dtype=torch.float64).reshape(cells[2], cells[1], cells[0])
    kp = F.pad(kc[None, None], (1, 1, 1, 1, 1, 1))
    ones = F.pad(torch.ones_like(kc)[None, None], (1, 1, 1, 1, 1, 1))
    box = torch.ones(1, 1, 2, 2, 2, dtype=torch.float64)
    f = [torch.log(F.conv3d(kp, box) / F.conv3d(ones, box))]
    w1 = torch.tensor([0.25, 0.5, 0.25], dtype=torch.float64)
    Rw = (w1[:, None, None] * w1[None, :, None] * w1[None, None, :])[None, None]

    def R(x):
        c = x.shape[1]
        return F.conv3d(x, Rw.repeat(c, 1, 1, 1, 1), stride=2, padding=1, groups=c)

    if coarse_start:
        f = [R(f[0])]
    for _ in range(1, levels):
        f.append(R(f[-1]))
    s = [torch.sigmoid(F.conv3d(f[l], G[l], bias=Bs[l], padding=1)) for l in range(levels)]
    dsq = torch.sqrt(dinv)
    xf = torch.zeros(nlat, dtype=torch.float64)
    xf[node_of_gid] = dsq * r_gid
    xf = xf.reshape(1, 1, N[2], N[1], N[0]).requires_grad_(True)
    x0 = R(xf) if coarse_start else xf
    hs, x = [], x0
    for l in range(levels):
        if l > 0:
            x = R(hs[-1])
        hs.append(F.conv3d(x, W[l], padding=1) * s[l])
    q = 0.5 * sum((h * h).sum() for h in hs)
    y, = torch.autograd.grad(q, xf, create_graph=True)
    return dinv * r_gid + dsq * y.reshape(-1)[node_of_gid]


def small_system(be, seed=41):
    pb = make_problem(3, (8, 8, 8), (2, 2, 2), 1, seed=seed)
    model, V, op = build(be, pb)
    A = torch.tensor(global_matrix(op).toarray(), dtype=torch.float64)
    return pb, V, op, A


@pytest.mark.parametrize("levels,cs", [(1, False), (3, False), (4, False), (1, True), (3, True)])
def test_network_gradient_matches_pytorch(levels, cs):
    import gridap_gb300 as G
    from gridap_gb300.learned import LearnedPreconditioner
    be = G.GB300Backend(0)
    try:
        pb, V, op, A = small_system(be)
        net = LearnedPreconditioner(op.matrix, seed=7, levels=levels, coarse_start=cs)
        assert net.num_params == C8 * TAPS + (levels - 1) * C8 * C8 * TAPS + levels * (C8 * TAPS + C8)
        n = V.num_free_dofs()
        rng = np.random.default_rng(5)
        r = rng.standard_normal((2, n)).astype(np.float32)
        e = rng.standard_normal((2, n)).astype(np.float32)
        rd, ed = torch.tensor(r, device="cuda"), torch.tensor(e, device="cuda")
        loss_gpu, grad_gpu = net.gradient(rd, ed)
        z_gpu = net.apply(rd[0].contiguous()).cpu().numpy()
        # PyTorch CPU restatement
        dinv = 1.0 / torch.diagonal(A)
        node_of_gid = torch.tensor(gid_to_node(V))
        params = torch.tensor(net.get_params().astype(np.float64), requires_grad=True)
        total = 0.0
        for b in range(2):
            z = torch_net(params, pb.kappa, pb.n, torch.tensor(r[b], dtype=torch.float64), node_of_gid, dinv, levels,
                          cs)
            if b == 0:
                assert np.abs(z.detach().numpy() - z_gpu).max() <= 1e-4 * np.abs(z_gpu).max()
            ev = torch.tensor(e[b], dtype=torch.float64)
            d = z - ev
            total = total + (d @ (A @ d)) / (ev @ (A @ ev))
        total.backward()
        loss_cpu = total.item() / 2
        assert abs(loss_gpu - loss_cpu) <= 1e-4 * abs(loss_cpu)
        gref = params.grad.numpy()
        rel = np.linalg.norm(grad_gpu - gref) / np.linalg.norm(gref)
        assert rel <= 2e-3, rel
        net.close()
    finally:
        be.close()


@pytest.mark.parametrize("cs", [False, True])
def test_network_is_symmetric_positive_definite(cs):
    """<r1, M r2> = <M r1, r2> and <r, M r> > 0 for the device network, also with
    parameters far from the initial ones."""
    import gridap_gb300 as G
    from gridap_gb300.learned import LearnedPreconditioner
    be = G.GB300Backend(0)
    try:
        pb, V, op, A = small_system(be, seed=43)
        net = LearnedPreconditioner(op.matrix, seed=11, levels=3, coarse_start=cs)
        rng = np.random.default_rng(9)
        net.set_params(rng.standard_normal(net.num_params).astype(np.float32) * 0.5)
        n = V.num_free_dofs()
        r = torch.tensor(rng.standard_normal((3, n)), device="cuda", dtype=torch.float32)
        z = [net.apply(r[i].contiguous()).double() for i in range(3)]
        rr = r.double()
        a, b = torch.dot(rr[0], z[1]).item(), torch.dot(z[0], rr[1]).item()
        scale = (torch.linalg.vector_norm(rr[0]) * torch.linalg.vector_norm(z[1])).item()
        assert abs(a - b) <= 1e-5 * scale, (a, b)
        for i in range(3):
            assert torch.dot(rr[i], z[i]).item() > 0
        net.close()
    finally:
        be.close()


@pytest.mark.parametrize("levels,cs", [(1, False), (2, False), (3, False), (4, False), (1, True), (3, True)])
def test_tiled_application_matches_training_kernels(levels, cs):
    """The solver's tiled application (fused gather, gates and output) against the
    training kernels on a lattice with partial tiles in every direction, with
    parameters large enough that the learned term dominates D^-1 r."""
    import ctypes as C
    import gridap_gb300 as G
    from gridap_gb300 import _lib as L
    from gridap_gb300.learned import LearnedPreconditioner
    be = G.GB300Backend(0)
    try:
        pb = make_problem(3, (24, 16, 20), (2, 2, 1), 1, seed=47, domain=(0.0, 1.5, 0.0, 1.0, 0.0, 1.25))
        model, V, op = build(be, pb)
        net = LearnedPreconditioner(op.matrix, seed=13, levels=levels, coarse_start=cs)
        rng = np.random.default_rng(21)
        net.set_params(rng.standard_normal(net.num_params).astype(np.float32) * 0.3)
        n = V.num_free_dofs()
        r = torch.tensor(rng.standard_normal(n), device="cuda", dtype=torch.float32)
        z_fast = net.apply(r)
        z_ref = torch.empty_like(r)
        L.call("gd_learned_apply_reference", net.handle, C.c_void_p(r.data_ptr()), C.c_void_p(z_ref.data_ptr()))
        dinv_r = z_ref.abs().max().item()
        assert torch.isfinite(z_fast).all()
        assert (z_fast - z_ref).abs().max().item() <= 1e-5 * dinv_r
        net.close()
    finally:
        be.close()


def test_training_on_solver_pairs_beats_jacobi(tmp_path):
    """Train on pairs generated by the solver for a few coefficient fields, then solve a
    field the network has not seen: the learned flexible CG needs fewer iterations than
    Jacobi-preconditioned CG to the same FP64 relative residual."""
    import gridap_gb300 as G
    from gridap_gb300.learned import LearnedPreconditioner, solver_pairs
    from gridap_gb300.synthetic import lognormal_kappa
    be = G.GB300Backend(0)
    try:
        cells = (24, 24, 24)
        pb = make_problem(3, cells, (2, 2, 2), 1, seed=None)
        pb.kappa = lognormal_kappa(cells, sigma=1.5, corr_len=0.05, seed=100)
        model, V, op = build(be, pb)
        net = LearnedPreconditioner(op.matrix, seed=1)
        rng = np.random.default_rng(0)
        n = V.num_free_dofs()
        fields = [lognormal_kappa(cells, sigma=1.5, corr_len=0.05, seed=200 + s) for s in range(6)]
        dO = G.Measure(G.Triangulation(model), 2)
        data = []
        for kap in fields:
            op.assem.numeric(G.integral_grad_grad(kap, dO), G.integral_source(1.0, dO))
            b = torch.tensor(rng.standard_normal(n), device="cuda", dtype=torch.float64)
            data.append((kap, *solver_pairs(op.matrix, b, ks=(2, 8, 32))))
        losses = []
        for epoch in range(25):
            for kap, r, e in data:
                op.assem.numeric(G.integral_grad_grad(kap, dO), G.integral_source(1.0, dO))
                losses.append(net.train_step(r, e, lr=3e-3))
        first, last = np.mean(losses[:len(data)]), np.mean(losses[-len(data):])
        assert last < 0.7 * first, (first, last)
        # unseen field
        kap = lognormal_kappa(cells, sigma=1.5, corr_len=0.05, seed=999)
        op.assem.numeric(G.integral_grad_grad(kap, dO), G.integral_source(1.0, dO))
        xj = op.matrix.solve(rtol=1e-8, method="mixed_ir")
        it_j = op.matrix.last_stats.iterations
        xl, st, fallback = net.solve(rtol=1e-8)
        assert st.converged and not fallback
        assert st.iterations < it_j, (st.iterations, it_j)
        assert np.abs(xl - xj).max() <= 1e-6 * np.abs(xj).max()
        # versioned parameter file round trip
        path = tmp_path / "net.gdlp"
        net.save(path)
        p0 = net.get_params()
        net.set_params(np.zeros_like(p0))
        net.load(path)
        assert np.array_equal(net.get_params(), p0)
        net.close()
    finally:
        be.close()
