"""CPU checks of bench.py's TiO2 per-iteration mode with a stand-in for the library context: each form
runs in its own context (so each pays its own one-time set-up and first-iteration products), the
first mixed iteration is kept apart from the later FP32 ones, and the evaluation model adds the parts
as documented."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class _FakeContext:
    """Iteration kinds as the library reports them for the options the per-iteration mode passes;
    iteration k of a call takes (k + 1) s, plus 100 s for the first iteration of a context."""
    created = []

    def __init__(self, device):
        self.norb = 0
        self.kinds = []
        self.calls = 0
        _FakeContext.created.append(self)

    def set_model(self, model):
        pass

    def set_geometry(self, coords, species):
        self.norb = 6 * len(species)

    def scc(self, o):
        from dftbplus_gb300 import binding
        mi = o.max_iter
        if o.precision == binding.PREC_FP64:
            k = [binding.PREC_FP64] * mi
        elif o.mixed_switch_tol > 1.0:
            k = [binding.PREC_MIXED, binding.PREC_FP64, binding.ITER_PERTURB, binding.ITER_PERTURB,
                 binding.PREC_FP64][:mi]
        else:
            k = [binding.PREC_MIXED] * (mi - 1) + [binding.PREC_FP64]
        self.kinds = k
        self.first = self.calls == 0
        self.calls += 1
        return {"converged": mi > 10, "energies": {"EMermin": -1.0}}

    def gradients(self):
        return None

    def scc_history(self):
        ms = (np.arange(1, len(self.kinds) + 1) * 1000.0)
        if self.first:
            ms[0] += 100000.0
        return {"precision": np.array(self.kinds), "ms": ms}

    def close(self):
        pass


def test_per_iteration_forms_use_own_contexts(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    from dftbplus_gb300 import binding, synth
    _FakeContext.created = []
    monkeypatch.setattr(binding, "Context", _FakeContext)
    monkeypatch.setattr(bench, "_workload", lambda name: (None, np.zeros((4, 3)), np.zeros(4, dtype=int)))
    monkeypatch.setattr(synth, "anatase_cluster", lambda nti: (np.zeros((nti, 3)), np.zeros(nti, dtype=int)))
    monkeypatch.setattr(sys, "argv", ["bench.py", "--config", "tio2", "--per-iteration"])
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    # two full-size contexts (FP64, mixed) plus one per convergence sphere
    assert len(_FakeContext.created) == 4
    per = line["mixed"]["iteration_s"]
    assert per["fp32_first"] == pytest.approx(101.0)   # first iteration of the mixed context
    assert per["fp32"] == pytest.approx(1.0)           # a later FP32 iteration (second call)
    assert per["fp64_class"] == pytest.approx(2.0)
    assert per["perturbative"] == pytest.approx(3.0)
    assert line["fp64"]["iteration_s"] == [pytest.approx(101.0), pytest.approx(2.0)]
    m = line["evaluation_model"]
    conv = line["convergence"][-1]
    n64 = conv["fp64"]["iterations"]
    bk = conv["mixed"]["by_kind"]
    t64 = line["fp64"]["set_geometry_s"] + 101.0 + (n64 - 1) * 2.0 + line["fp64"]["gradients_s"]
    tmx = (line["mixed"]["set_geometry_s"] + 101.0 + (bk.get("fp32", 0) - 1) * 1.0
           + bk.get("fp64_class", 0) * 2.0 + bk.get("perturbative", 0) * 3.0 + line["mixed"]["gradients_s"])
    assert m["fp64_s"] == pytest.approx(t64)
    assert m["mixed_s"] == pytest.approx(tmx)
    assert m["mixed_vs_fp64"] == pytest.approx(t64 / tmx)
