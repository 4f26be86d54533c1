"""Batches of realisations (gethi_gpu_run_batch): one CUDA graph over several
configurations must give the maps of the same seeds run one at a time; the
launch-shape autotuner must keep the results."""
import numpy as np
import pytest

from conftest import load_case
from test_gpu_parity import gh, params_for_case  # noqa: F401  (fixture)

NU21 = 1420.40575177


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [True, False])
def test_run_batch_matches_single_runs(gh, graph):  # noqa: F811
    ctxs = [gh.GetHI(params_for_case(gh, load_case(name), velocity_mode="spectral"))
            for name in ("case_irr32", "case_reg24")]
    jobs = [(0, 11), (1, 12), (0, 13), (1, 14), (0, 15)]
    maps, st = gh.run_batch(ctxs, jobs, graph=graph)
    assert st["kernel_launches"] > 0
    if graph:
        assert st["graph_nodes"] >= st["kernel_launches"]
    for (k, seed), m in zip(jobs, maps):
        ctxs[k].set_seed(seed)
        ref = ctxs[k].run()
        assert np.abs(ref).max() > 0
        assert _rel(m, ref) < 1e-6  # only the FP32 accumulation order may differ
    # different seeds give different maps
    assert _rel(maps[0], maps[2]) > 1e-2
    for c in ctxs:
        c.free()


@pytest.mark.gpu
def test_autotune_keeps_results(gh):  # noqa: F811
    p = gh.make_params(pk_filename="EH", frequencies_filename="", nu_min=NU21 / 1.5, nu_max=NU21 / 1.2, n_nu=16,
                       n_side=64, n_grid=128, l_box=2000.0, seed=4000, do_rsd=1, velocity_mode="spectral",
                       gaussianise=1)
    ctx = gh.GetHI(p)
    ctx.set_seed(4000)
    ref = ctx.run()
    tuned = ctx.autotune()
    assert tuned["tile_depth"] in (4, 8, 16) and tuned["column_variant"] in (0, 1)
    assert tuned["ms_per_realisation"] > 0
    ctx.set_seed(4000)
    got = ctx.run()
    assert np.abs(ref).max() > 0
    # a different column tile changes FP32 rounding of the fields, so a few samples near a
    # pixel or shell edge may move
    assert _rel(got, ref) < 1e-3
    ctx.free()


@pytest.mark.gpu
def test_run_async_pipeline_matches_run(gh):  # noqa: F811
    """Pipelined realisations (two device map buffers, copies on a second stream)
    give the maps of the same seeds run one at a time."""
    import torch
    ctx = gh.GetHI(params_for_case(gh, load_case("case_irr32"), velocity_mode="spectral"))
    shape = (ctx.n_nu, ctx.npix)
    outs = [torch.zeros(shape, dtype=torch.float32).pin_memory() for _ in range(2)]
    dev = torch.zeros(shape, dtype=torch.float32, device="cuda")
    seeds = [31, 32, 33, 34]
    got = {}
    for i, s in enumerate(seeds):
        ctx.set_seed(s)
        if i == 3:
            ctx.run_async(dev.data_ptr())  # device destination
        else:
            if i == 2:
                ctx.wait()  # buffer 0 is reused: collect the first result
                got[seeds[0]] = outs[0].numpy().copy()
            ctx.run_async(outs[i % 2].data_ptr())
    ctx.wait()
    got[seeds[1]] = outs[1].numpy().copy()
    got[seeds[2]] = outs[0].numpy().copy()
    got[seeds[3]] = dev.cpu().numpy()
    for s in seeds:
        ctx.set_seed(s)
        ref = ctx.run()
        assert np.abs(ref).max() > 0
        assert _rel(got[s], ref) < 1e-6
    ctx.free()
