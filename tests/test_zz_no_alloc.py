"""pd_apply_operator_noalloc, the entry point for callers that cannot call
cudaMalloc (a host application that owns all device memory and hands this
library pointers into its own pool, or a time-critical loop that must not
allocate).  Its output must equal pd_apply_operator's on the same view and
vectors, on two calls in a row (the static scratch is reused and keeps the
previous call's contents).  This file is collected last on purpose."""
import gc

import numpy as np
import pytest


pytestmark = pytest.mark.gpu

TOL = {0: 1e-5, 1: 1e-9}   # mixed / FP64, the tolerances of the parity tests


def _vectors(pdgb, sim, seed):
    import torch
    v = sim.operator_view()
    dt = torch.float32 if v.precision == pdgb.PRECISION_MIXED else torch.float64
    g = torch.Generator(device="cpu").manual_seed(seed)
    x = torch.zeros((v.n, 4), dtype=dt)
    x[:, :3] = torch.randn((v.n, 3), generator=g, dtype=torch.float64).to(dt)
    return v, x.cuda()


@pytest.mark.parametrize("blocks", [None, 0, 1])
@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_apply_operator(pdgb, scenes, precision, blocks):
    """blocks None: the view's own grid; 0: the automatic grid (rows per
    block from the lanes, at most 4096 blocks); 1: one block striding over
    every row."""
    import torch
    sc = scenes.reference_block(n_side=9, integrator=pdgb.NEWMARK_BETA, adaptive=1, expansion=300.0)
    sc.opt.precision = precision
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    sim.advance(32)
    v, x = _vectors(pdgb, sim, 3)
    if blocks is not None:
        v.blocks = blocks
    y_ref = torch.full_like(x, float("nan"))
    dot_ref = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    sim.synchronize()
    torch.cuda.synchronize()
    sim.apply_operator(x.data_ptr(), y_ref.data_ptr(), dot_ref.data_ptr())
    sim.synchronize()
    stream = sim.stream_handle()
    for call in range(2):
        y = torch.full_like(x, float("nan"))
        dot = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        pdgb.apply_operator_noalloc(v, x.data_ptr(), y.data_ptr(), dot.data_ptr(), stream)
        sim.synchronize()
        a = y[:, :3].double().cpu().numpy()
        b = y_ref[:, :3].double().cpu().numpy()
        assert np.isfinite(a).all()
        assert np.abs(a - b).max() <= TOL[precision] * np.abs(b).max(), f"call {call}"
        assert abs(dot.item() - dot_ref.item()) <= TOL[precision] * abs(dot_ref.item()), f"call {call}"


def test_noalloc_rejects_more_blocks_than_the_scratch_holds(pdgb, scenes):
    import torch
    sc = scenes.reference_block(n_side=6)
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    v, x = _vectors(pdgb, sim, 4)
    y = torch.zeros_like(x)
    v.blocks = 4097
    with pytest.raises(pdgb.PdError) as e:
        pdgb.apply_operator_noalloc(v, x.data_ptr(), y.data_ptr(), None, sim.stream_handle())
    assert e.value.status == 1 and "4096" in str(e.value)


def test_noalloc_allocates_nothing(pdgb, scenes):
    """Repeated calls leave the device's free memory unchanged (measured after
    a first call, which loads the library's module and resolves the scratch)."""
    import torch
    sc = scenes.reference_block(n_side=8)
    sim = scenes.make_simulator(sc)
    sim.makeReady()
    v, x = _vectors(pdgb, sim, 5)
    v.blocks = 0
    y = torch.zeros_like(x)
    dot = torch.zeros((1,), dtype=torch.float64, device="cuda")
    stream = sim.stream_handle()
    torch.cuda.synchronize()
    pdgb.apply_operator_noalloc(v, x.data_ptr(), y.data_ptr(), dot.data_ptr(), stream)
    sim.synchronize()
    # tensors of earlier tests still waiting for the cycle collector would
    # otherwise be released in the middle of the measurement
    gc.collect()
    free0, _ = torch.cuda.mem_get_info()
    torch_bytes0 = torch.cuda.memory_allocated()
    for _ in range(20):
        pdgb.apply_operator_noalloc(v, x.data_ptr(), y.data_ptr(), dot.data_ptr(), stream)
    sim.synchronize()
    gc.collect()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_allocated() == torch_bytes0
