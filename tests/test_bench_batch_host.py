"""The batch bench arm's host logic on CPU, against a stub of the C ABI (no GPU).

bench.run_batch drives hyperfox_gb300.batch (group tolerances, per-group timing marks,
kernel-time collection, the host-buffer step, the line's keys). Here every device call
of the C ABI is replaced by a stub that returns success, with fixed timings and
iteration counts, while the host-only entry points (topology, high-order nodes) stay
the library's own. The test checks that the arm runs end to end and prints the
contract's keys with consistent arithmetic; it measures nothing.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class _StubLib:
    """Device entry points return 0; hfx_kernel_time reports 10 launches / 1.5 ms,
    hfx_elapsed_ms 2 ms, hfx_elapsed_between 0 ms to a start mark and 2 ms to an end mark
    (every group from 0 to 2 ms), hfx_solve 7 iterations. Host entry points are the
    library's."""

    def __init__(self, real):
        self.real = real

    def __getattr__(self, name):
        if name.startswith(("hfx_mesh_", "hfx_refel")):
            return getattr(self.real, name)

        def call(*a):
            if name == "hfx_kernel_time":
                a[2]._obj.value, a[3]._obj.value = 10, 1.5
            elif name == "hfx_elapsed_ms":
                a[3]._obj.value = 2.0
            elif name == "hfx_elapsed_between":
                a[4]._obj.value = 2.0 if a[3] == 1 else 0.0
            elif name == "hfx_solve":
                a[3]._obj.iterations = 7
            return 0
        return call


class _StubContext:
    def __init__(self, device=0):
        from hyperfox_gb300 import capi
        self.L = capi.load()  # the stub while the test runs
        self.h = 1

    def _chk(self, rc, what):
        assert rc == 0, what

    def upload_mesh(self, dim, order, coords, cells, topology=None):
        from hyperfox_gb300 import capi
        self.re = capi.refel(dim, order)
        self.nCells, self.nFaces = cells.shape[0], topology[2].shape[0]
        self.ndofs = self.nFaces * self.re["nNodesFace"]
        self.lenU, self.lenQ = self.re["nNodes"], dim * self.re["nNodes"]
        self.nnz = self.ndofs * 5 * self.re["nNodesFace"]

    def set_tau(self, t):
        assert t.shape[0] == self.nFaces

    def set_dirichlet(self, g):
        assert g.shape[0] == self.nFaces

    def set_kappa(self, k, layout=1):
        assert k.shape[0] == self.nCells

    def set_source(self, *a):
        pass

    def assemble(self, *a):
        pass

    def get_state(self):
        return np.zeros((self.nCells, self.lenU)), np.zeros((self.nCells, self.lenQ)), np.zeros(self.ndofs)

    def close(self):
        pass


@pytest.mark.parametrize("serial", [False, True])
def test_batch_arm_runs_on_a_stub_abi(monkeypatch, serial):
    import types

    import torch
    sys.path.insert(0, ROOT)
    import bench
    from hyperfox_gb300 import capi
    stub = _StubLib(capi.load())
    monkeypatch.setattr(capi, "load", lambda *a: stub)
    monkeypatch.setattr(capi, "Context", _StubContext)
    monkeypatch.setattr(torch.cuda, "set_device", lambda *a: None)
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a: None)
    empty = torch.empty
    monkeypatch.setattr(torch, "empty", lambda *a, **k: empty(*a, **{x: v for x, v in k.items() if x != "pin_memory"}))
    monkeypatch.setitem(bench.CONFIGS, "stub", dict(dim=2, batch=dict(count=12, seed=3, min_elements=20,
                                                                      max_elements=400), cpu_budget=300,
                                                   desc="stub"))
    args = types.SimpleNamespace(config="stub", rtol=1e-8, precision="mixed", precond="twolevel", inner_rtol=1e-2,
                                 coarse_rtol=0.3, coarse_degree=8, warmup=1, steps=2, batch_serial=serial)
    res, B = bench.run_batch(args, 1, 0, 0)
    groups = len(B.groups)
    assert groups > 1
    assert res["config"]["elements"] == B.nCells and res["config"]["problems"] == 12
    # serial: the groups' 2 ms of stub events add up; concurrent: every group runs from 0 to
    # 2 ms, so a step spans 2 ms
    step = 2.0 * groups if serial else 2.0
    assert res["ms_per_step"] == pytest.approx(step)
    assert res["value"] == pytest.approx(B.nCells / (step / 1e3))
    for key in ("metric", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling", "dtype", "roofline",
                "clocks", "e2e", "gpu_launches"):
        assert key in res, key
    assert res["roofline"]["bound"] == "hbm" and res["roofline"]["unit"] == "GB/s"
    assert res["e2e"]["h2d_bytes_per_step"] > 0 and res["e2e"]["d2h_bytes_per_step"] > 0
    assert res["gpu_launches"] == 9 * 10 * groups
    assert set(res["group_ms_alone"]) == {str(q) for q in B.groups}
