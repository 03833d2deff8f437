"""SAH of the GPU optimizer against the reference's own optimizers at equal iteration count, on the
full-size scenes (the reference's outputs are committed in tests/golden/ref_pin.npz, written by
tests/golden/make_ref_golden.py from the reference's Bittner13.cpp and Bittner13Par.cpp).

The bar is 0.5% relative to Bittner13Par, the reference's CPU form of the same chunked algorithm
(32 chunks of 1% per iteration, conflicting reinsertions of a chunk skipped): the GPU runs that
algorithm with its own deterministic conflict rule and its batched search, which picks the same
positions as the reference's heap search up to ties. Against the sequential Bittner13, which
never skips a reinsertion, the gap is reported and bounded looser (the chunked form trades a
little SAH per iteration for parallelism, in the reference as here).
"""
from pathlib import Path

import numpy as np
import pytest

from bvhtest_gb300 import scenes

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
TOL_PAR = 0.005
TOL_SEQ = 0.01


def _large(gpu, vert, faces):
    import torch
    n = faces.shape[0]
    v = torch.from_numpy(vert).cuda()
    f = torch.from_numpy(faces.view(np.int32)).cuda()
    b = gpu.LBVH(n, 63, "karras")
    nodes = b.build(v, f)
    torch.cuda.synchronize()
    assert b.errors() == 0
    b.close()
    return nodes, 2 * n - 1


def _check(gpu, key, vert, faces, checkpoints):
    import torch
    pin = np.load(GOLDEN / "ref_pin.npz")
    nodes, nn = _large(gpu, vert, faces)
    del vert, faces
    sah0 = gpu.calc_sah(nodes, 0, nn)
    assert sah0 == pytest.approx(float(pin[f"{key}_start_sah"]), rel=1e-9)  # the same LBVH
    opt = gpu.Bittner13GPU(nodes, num_nodes=nn)
    done = 0
    report = []
    for it in checkpoints:
        opt.run(it - done)
        done = it
        torch.cuda.synchronize()
        sah = gpu.calc_sah(nodes, 0, nn)
        par, seq = float(pin[f"{key}_par_sah"][it]), float(pin[f"{key}_seq_sah"][it])
        report.append((it, sah, par, seq))
        assert abs(sah / par - 1.0) <= TOL_PAR, report
        assert sah <= seq * (1.0 + TOL_SEQ), report
    opt.close()
    return report


def test_large_scene_sah_vs_reference_optimizers(gpu):
    """4,194,304 triangles, 63-bit karras LBVH, 200 iterations at 1%."""
    vert, faces = scenes.large_scene()
    _check(gpu, "c2", vert, faces, (10, 50, 100, 150, 200))


def test_stress_scene_sah_vs_reference_optimizers(gpu):
    """33,554,432 triangles, 63-bit karras LBVH; the reference's optimizers were run for 20
    iterations (the sequential one takes minutes per iteration at this size)."""
    pin = np.load(GOLDEN / "ref_pin.npz")
    if "c5_par_sah" not in pin:
        pytest.skip("no stress-scene fixture")
    vert, faces = scenes.stress_scene()
    _check(gpu, "c5", vert, faces, (5, 10, 20))
