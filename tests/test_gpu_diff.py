"""Differentiable form: dE/dR, dE/d(SK grid values) and dE/dU from the adjoint kernels, checked
against central finite differences of the GPU energy (steps: 1e-4 Bohr for positions, 1e-6 relative
for table values and U) and, for positions, against the oracle's analytic gradients."""
import numpy as np
import pytest

from oracle import dftb_oracle as O

pytestmark = pytest.mark.gpu

TOL = dict(kT=1e-3, scc_tol=1e-10)


def _energy(ctx, packed, coords, species):
    from dftbplus_gb300 import binding
    ctx.set_model_packed(packed)
    ctx.set_geometry(coords, species)
    r = ctx.scc(binding.default_opts(**TOL))
    assert r["converged"]
    return r["energies"]["EMermin"]


def _setup(water_model, n_mol, radius, seed):
    from dftbplus_gb300 import binding, synth
    c, s = synth.water_cluster(n_mol, radius, seed)
    ctx = binding.Context(0)
    base = water_model.pack()
    e0 = _energy(ctx, base, c, s)
    g = ctx.gradients()
    gh, go, gu = ctx.grad_params()
    return ctx, base, c, s, e0, g, gh, go, gu


def test_positions_fd_and_oracle(gpu_lib, water_model):
    ctx, base, c, s, e0, g, *_ = _setup(water_model, 6, 5.0, 7)
    gref = O.gradients(O.System(water_model, c, s), O.run_scc(O.System(water_model, c, s), kt=1e-3, scc_tol=1e-10))
    assert np.max(np.abs(g - gref)) < 1e-8
    h = 1e-4
    for (k, a) in [(0, 0), (1, 3), (2, 7), (0, 11)]:
        cp, cm = c.copy(), c.copy()
        cp[k, a] += h
        cm[k, a] -= h
        fd = (_energy(ctx, base, cp, s) - _energy(ctx, base, cm, s)) / (2 * h)
        assert abs(fd - g[k, a]) < 1e-6, (k, a, fd, g[k, a])
    ctx.close()


def test_hubbard_fd(gpu_lib, water_model):
    ctx, base, c, s, e0, g, gh, go, gu = _setup(water_model, 8, 6.3, 11)
    for sp in range(len(gu)):
        u = base["hubbu"][sp]
        h = 1e-6 * u
        pp, pm = dict(base), dict(base)
        pp["hubbu"] = base["hubbu"].copy(); pp["hubbu"][sp] = u + h
        pm["hubbu"] = base["hubbu"].copy(); pm["hubbu"][sp] = u - h
        fd = (_energy(ctx, pp, c, s) - _energy(ctx, pm, c, s)) / (2 * h)
        assert abs(fd - gu[sp]) < 1e-6 + 1e-5 * abs(gu[sp]), (sp, fd, gu[sp])
    ctx.close()


@pytest.mark.parametrize("kind", ["sk_ham", "sk_over"])
def test_sk_table_fd(gpu_lib, water_model, kind):
    """Entries with the largest gradients, including grid points that only reach the energy through
    the 5th-order tail beyond the last grid point (pairs at 12-13 Bohr in a 16-molecule cluster)."""
    ctx, base, c, s, e0, g, gh, go, gu = _setup(water_model, 16, 8.0, 4)
    grad = gh if kind == "sk_ham" else go
    picks = list(np.argsort(-np.abs(grad))[:5])
    # the last grid point of every table column (tail window): one with a non-zero gradient
    rows, nint = base["sk_rows"], base["sk_nint"]
    offs = np.concatenate([[0], np.cumsum(rows * nint)])
    tail = [offs[p] + k * rows[p] + rows[p] - 1 for p in range(len(rows)) for k in range(nint[p])]
    tail = [t for t in tail if abs(grad[t]) > 1e-7]
    assert tail, "no pair in the tail region"
    picks.append(max(tail, key=lambda t: abs(grad[t])))
    for idx in picks:
        y = base[kind][idx]
        h = 1e-6 * max(abs(y), 1e-3)
        pp, pm = dict(base), dict(base)
        pp[kind] = base[kind].copy(); pp[kind][idx] = y + h
        pm[kind] = base[kind].copy(); pm[kind][idx] = y - h
        fd = (_energy(ctx, pp, c, s) - _energy(ctx, pm, c, s)) / (2 * h)
        assert abs(fd - grad[idx]) < 1e-6 + 2e-4 * abs(grad[idx]), (kind, idx, fd, grad[idx])
    ctx.close()


def test_autograd_function(gpu_lib, water_model):
    torch = pytest.importorskip("torch")
    from dftbplus_gb300 import binding, synth
    from dftbplus_gb300.autograd import DftbEnergy
    c, s = synth.water_cluster(4, 4.0, 2)
    eng = DftbEnergy(water_model, s, kT=1e-3, scc_tol=1e-10)
    sk_h, sk_o, hub = (t.requires_grad_() for t in eng.parameters())
    x = torch.tensor(c, dtype=torch.float64, requires_grad=True)
    e = eng(x, sk_h, sk_o, hub)
    e.backward()
    ctx = binding.Context(0)
    e_ref = _energy(ctx, water_model.pack(), c, s)
    assert abs(e.item() - e_ref) < 1e-12
    gh, go, gu = ctx.grad_params()
    assert np.allclose(x.grad.numpy(), ctx.gradients(), atol=1e-12)
    assert np.allclose(sk_h.grad.numpy(), gh, atol=1e-12)
    assert np.allclose(sk_o.grad.numpy(), go, atol=1e-12)
    assert np.allclose(hub.grad.numpy(), gu, atol=1e-12)
    ctx.close()
    eng.close()


def test_water128_differentiation(gpu_lib, water_model):
    """(H2O)128 in FP64: forces plus parameter gradients, spot-checked by central differences."""
    ctx, base, c, s, e0, g, gh, go, gu = _setup(water_model, 128, 20.0, 128)
    for sp in range(len(gu)):
        u = base["hubbu"][sp]
        h = 1e-5 * u
        pp, pm = dict(base), dict(base)
        pp["hubbu"] = base["hubbu"].copy(); pp["hubbu"][sp] = u + h
        pm["hubbu"] = base["hubbu"].copy(); pm["hubbu"][sp] = u - h
        fd = (_energy(ctx, pp, c, s) - _energy(ctx, pm, c, s)) / (2 * h)
        assert abs(fd - gu[sp]) < 1e-5 + 1e-5 * abs(gu[sp]), (sp, fd, gu[sp])
    idx = int(np.argmax(np.abs(gh)))
    y = base["sk_ham"][idx]
    h = 1e-5 * abs(y)
    pp, pm = dict(base), dict(base)
    pp["sk_ham"] = base["sk_ham"].copy(); pp["sk_ham"][idx] = y + h
    pm["sk_ham"] = base["sk_ham"].copy(); pm["sk_ham"][idx] = y - h
    fd = (_energy(ctx, pp, c, s) - _energy(ctx, pm, c, s)) / (2 * h)
    assert abs(fd - gh[idx]) < 1e-4 * abs(gh[idx]), (idx, fd, gh[idx])
    cp, cm = c.copy(), c.copy()
    cp[2, 100] += 1e-4
    cm[2, 100] -= 1e-4
    fd = (_energy(ctx, base, cp, s) - _energy(ctx, base, cm, s)) / 2e-4
    assert abs(fd - g[2, 100]) < 1e-6
    ctx.close()
