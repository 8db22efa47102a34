"""Batched serving: many uneven Poisson / elasticity solves in one batch.  Every
problem's FP64 residual is checked with the oracle operator on its own mesh, and
the graph-replayed solve is compared with the eagerly launched one."""

import numpy as np
import pytest

import oracle as O
from sfem_gb300 import capi
from sfem_gb300.batch import BatchSolver, ConcurrentBatchSolver, ProblemSpec
from sfem_gb300.mesh import SSMesh

pytestmark = pytest.mark.gpu

# uneven sizes and levels; even edges also get hex8 levels below their macro grid
PROBLEMS = [ProblemSpec("poisson", 4, 2, 11), ProblemSpec("poisson", 6, 2, 12), ProblemSpec("poisson", 3, 4, 13),
            ProblemSpec("poisson", 5, 3, 14), ProblemSpec("elasticity", 4, 2, 21), ProblemSpec("elasticity", 3, 3, 22),
            ProblemSpec("elasticity", 2, 4, 23), ProblemSpec("poisson", 2, 4, 15), ProblemSpec("poisson", 8, 2, 16),
            ProblemSpec("elasticity", 4, 4, 24)]


def _oracle_residual(p, b, x, perturb=0.1):
    m = SSMesh(p.n, p.n, p.n, p.level, perturb=perturb, seed=p.seed)
    L = p.level
    el = m.elements(L)
    corners = el[m.macro_corner_lidx(L)]
    dn = m.boundary_nodes("x0", L).astype(np.int64)
    if p.kind == "poisson":
        fff = O.fff_fill(corners, m.points)
        y = O.sshex8_laplacian_apply(L, el, fff, x)
        y[dn] = x[dn]
    else:
        adj, det = O.adjugate_fill(corners, m.points)
        y = O.linear_elasticity_apply(L, el, adj, det, 1.0, 10.0, x)
        for c in range(3):
            y[3 * dn + c] = x[3 * dn + c]
    return np.linalg.norm(b - y) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def batch(cuda):
    return BatchSolver(PROBLEMS, device=cuda, coarse_iterations=20)


def test_batch_solve_matches_oracle(cuda, batch):
    import torch

    b = batch.rhs()
    x = torch.zeros_like(b)
    rc, lat, its, sec = batch.solve(b, x)
    assert rc == 0, capi.last_error()
    assert (its >= 1).all() and (lat > 0).all() and lat.max() <= sec + 1e-9
    tr = batch.true_residuals(b, x)
    assert (tr <= 1.5e-10).all(), tr
    bh, xh = b.cpu().numpy(), x.cpu().numpy()
    for i, p in enumerate(batch.problems):
        s = slice(batch.dof_offsets[i], batch.dof_offsets[i + 1])
        res = _oracle_residual(p, bh[s], xh[s])
        assert res <= 2e-10, (p, res)


def test_batch_graph_matches_eager(cuda):
    import torch

    probs = PROBLEMS[:3] + PROBLEMS[4:6]
    xs = []
    for g in (False, True):
        bs = BatchSolver(probs, device=cuda, coarse_iterations=20, use_graph=g)
        b = bs.rhs()
        x = torch.zeros_like(b)
        rc, *_ = bs.solve(b, x)
        assert rc == 0, capi.last_error()
        xs.append(x)
    # same kernels in the same order; the element scatters use float atomics, so the
    # two runs agree to rounding, far inside the solve tolerance
    assert float(torch.linalg.vector_norm(xs[0] - xs[1])) <= 1e-8 * float(torch.linalg.vector_norm(xs[0]))


def test_batch_autotune_and_dot(cuda, batch):
    import torch

    b = batch.rhs()
    lib = capi.load()
    before = lib.sfem_gb300_set_laplacian_kernel(-1)
    table = batch.autotune(b, candidates=[(1024, 128, 8), (4096, 256, 8)], reps=1,
                           kernels={"laplacian": (-1, 8), "elasticity": (-1, 0)})
    assert any(g.spaces[-1].is_macro_coarse for g in batch.groups)
    # two Laplacian and two elasticity kernel candidates, then both launch shapes
    assert len(table) == 6 and all(t > 0 for *_, t in table)
    assert batch.tuned_kernels["laplacian"] in (-1, 8) and batch.tuned_kernels["elasticity"] in (-1, 0)
    assert batch.tuned in [c for c, k, _ in table if k == batch.tuned_kernels]
    # the process-wide kernel choice is restored after tuning
    assert lib.sfem_gb300_set_laplacian_kernel(before) == -1
    x = torch.zeros_like(b)
    rc, lat, its, sec = batch.solve(b, x)
    assert rc == 0, capi.last_error()
    assert (batch.true_residuals(b, x) <= 1.5e-10).all()
    # segmented dot against per-problem torch dots
    y = torch.randn_like(b)
    out = torch.zeros(batch.n_problems, dtype=torch.float64, device=cuda)
    capi.check(capi.load().sfem_gb300_batch_dot(batch.layout.ptr, capi.FLOAT64, capi.vp(b), capi.vp(y),
                                                capi.vp(out)), "batch_dot")
    ref = torch.stack([torch.dot(b[s0:s1], y[s0:s1]) for s0, s1 in
                       zip(batch.dof_offsets[:-1], batch.dof_offsets[1:])])
    torch.testing.assert_close(out, ref, rtol=1e-12, atol=1e-12)


def test_batch_staggered_release(cuda, batch):
    """Problems released one after another (reverse batch order over 60 ms): each joins at
    the first chunk boundary after its release, converges to 1e-10, its latency counts from
    its own release, and it takes the iterations it takes when all start together (to a
    chunk: the checks fall on chunk boundaries)."""
    import torch

    b = batch.rhs()
    x0 = torch.zeros_like(b)
    rc, _, its_all, _ = batch.solve(b, x0)
    assert rc == 0, capi.last_error()
    P = batch.n_problems
    release = np.linspace(0.06, 0.0, P)
    x = torch.zeros_like(b)
    rc, lat, its, sec = batch.solve(b, x, release=release)
    assert rc == 0, capi.last_error()
    assert (lat > 0).all() and (lat + release <= sec + 1e-9).all()
    assert (its >= 1).all() and np.abs(its - its_all).max() <= batch.check_every, (its, its_all)
    assert (batch.true_residuals(b, x) <= 1.5e-10).all()
    with pytest.raises(ValueError):
        batch.solve(b, x, release=release[:-1])


def test_concurrent_groups(cuda, batch):
    """One batched solver per group on its own stream, advanced by the non-blocking
    begin / step / poll driver: every problem converges to 1e-10 (oracle residual on its
    own mesh), with the iterations the lockstep batch takes (to a chunk), and no group
    waits for another's chunks."""
    import torch

    cs = ConcurrentBatchSolver(PROBLEMS, device=cuda, coarse_iterations=20)
    assert len(cs.subs) == len(batch.groups) and sorted(map(str, cs.problems)) == sorted(map(str, batch.problems))
    # the smallest group gets the highest stream priority level, the largest the lowest
    sizes = [s.n for s in cs.subs]
    assert cs.priority[int(np.argmin(sizes))] == max(cs.priority) > cs.priority[int(np.argmax(sizes))] == 0
    bs = cs.rhs()
    xs = [torch.zeros_like(b) for b in bs]
    lat, its, sec = cs.solve(bs, xs)
    assert (lat > 0).all() and lat.max() <= sec + 1e-9 and (its >= 1).all()
    assert (cs.true_residuals(bs, xs) <= 1.5e-10).all()
    b0 = batch.rhs()
    x0 = torch.zeros_like(b0)
    rc, _, its_lock, _ = batch.solve(b0, x0)
    assert rc == 0, capi.last_error()
    order = {str(p): i for i, p in enumerate(batch.problems)}
    its_lock = np.array([its_lock[order[str(p)]] for p in cs.problems])
    assert np.abs(its - its_lock).max() <= batch.check_every, (its, its_lock)
    for i in (0, len(cs.problems) - 1):
        k = next(j for j in range(len(cs.subs)) if cs.offsets[j] <= i < cs.offsets[j + 1])
        s = cs.subs[k]
        q = i - cs.offsets[k]
        sl = slice(s.dof_offsets[q], s.dof_offsets[q + 1])
        res = _oracle_residual(cs.problems[i], bs[k].cpu().numpy()[sl], xs[k].cpu().numpy()[sl])
        assert res <= 2e-10, (cs.problems[i], res)
