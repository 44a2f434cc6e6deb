"""Geometry from the host's neighbour list (the reference's nNeighbourSK / iNeighbour layout, cluster
case) instead of the GPU's own: the same half list gives the same H0, S, energies, charges and
forces bit for bit; a list with every atom pair (most beyond the SK cutoff) gives the same results;
indices outside the cluster are rejected."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _neighbour_arrays(c, cutoff, everything=False):
    """Reference-style half list: atom i lists the atoms j < i within the cutoff (or all j < i)."""
    xyz = np.asarray(c, dtype=np.float64).T
    n = len(xyz)
    rows = []
    for i in range(n):
        d = np.linalg.norm(xyz[:i] - xyz[i], axis=1)
        js = np.arange(i) if everything else np.nonzero(d <= cutoff)[0]
        rows.append(js[np.argsort(d[js], kind="stable")])   # nearest first, as the reference sorts them
    maxn = max(1, max(len(r) for r in rows))
    ineigh = np.full((n, maxn + 1), -1, dtype=np.int32)
    for i, r in enumerate(rows):
        ineigh[i, 0] = i
        ineigh[i, 1:1 + len(r)] = r
    return np.array([len(r) for r in rows], dtype=np.int32), ineigh


def _evaluate(ctx, kT=1e-3):
    from dftbplus_gb300 import binding
    H0 = ctx.matrix(0)
    S = ctx.matrix(1)
    res = ctx.scc(binding.default_opts(kT=kT, scc_tol=1e-7))
    return H0, S, res, ctx.gradients()


@pytest.mark.parametrize("everything", [False, True])
def test_host_neighbour_list_matches_gpu_list(gpu_lib, water_model, everything):
    from dftbplus_gb300 import binding, synth
    c, s = synth.water_cluster(32, 10.0, 1)
    ctx = binding.Context(0)
    ctx.set_model(water_model)
    ctx.set_geometry(c, s)
    ref = _evaluate(ctx)
    nneigh, ineigh = _neighbour_arrays(c, water_model.sk_cutoff(), everything)
    ctx.set_geometry_neighbours(c, s, nneigh, ineigh)
    got = _evaluate(ctx)
    ctx.close()
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    assert got[2]["n_iter"] == ref[2]["n_iter"]
    assert abs(got[2]["energies"]["EMermin"] - ref[2]["energies"]["EMermin"]) < 1e-12
    assert np.max(np.abs(got[2]["q_out"] - ref[2]["q_out"])) < 1e-12
    assert np.max(np.abs(got[3] - ref[3])) < 1e-12


def test_host_neighbour_list_rejects_images(gpu_lib, water_model):
    from dftbplus_gb300 import binding, synth
    c, s = synth.water_cluster(4, 3.5, 3)
    nneigh, ineigh = _neighbour_arrays(c, water_model.sk_cutoff())
    ineigh = ineigh.copy()
    ineigh[5, 1] = len(s) + 3          # a periodic image index
    ctx = binding.Context(0)
    ctx.set_model(water_model)
    with pytest.raises(binding.DftbGpuError) as e:
        ctx.set_geometry_neighbours(c, s, nneigh, ineigh)
    assert e.value.code == 1
    ctx.close()
