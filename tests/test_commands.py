"""The BVHTest command layer (JSON configs driving the commands) over libbvhgb.

CPU tests run configs made only of host commands (load, BVHImport, validate, BVHExport, writeData,
status); the GPU test runs the reference's pipeline load -> copyToGPU -> LBVH -> bittner13GPU ->
CUDATracer -> copyToHost -> validate -> BVHExport -> writeData and checks the files it writes
against the oracle.
"""
import ctypes as C
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

from bvhtest_gb300 import meshio, native, scenes

ROOT = Path(__file__).resolve().parent.parent
CLI = ROOT / "bvhtest_gb300" / "lib" / "bvhTest"


def _run(cfg_path):
    lib = native.load()
    lib.bvhgb_run_config.restype = C.c_int
    lib.bvhgb_run_config.argtypes = [C.c_char_p]
    return lib.bvhgb_run_config(str(cfg_path).encode())


def _config(tmp, cmds, name="t"):
    cfg = {"baseConfig": {"name": name, "verbose": False, "basePath": str(tmp), "input": ["scene"]},
           "commands": cmds}
    p = Path(tmp) / "cfg.json"
    p.write_text(json.dumps(cfg))
    return p


def test_cli_list_and_generate(tmp_path):
    native.load()
    out = subprocess.run([str(CLI), "list"], capture_output=True, text=True)
    assert out.returncode == 0
    for name in ("LBVH", "bittner13GPU", "CUDATracer", "copyToGPU", "copyToHost", "validate", "writeData"):
        assert name in out.stdout
    gen = subprocess.run([str(CLI), "generate", "-", "load", "LBVH", "bittner13GPU"], capture_output=True, text=True)
    cfg = json.loads(gen.stdout)
    opts = cfg["commands"][2]["options"]
    # the reference's option names and defaults (Bittner13GPU.hpp:28-37, OptimizerBase.cpp:28-33)
    assert opts["maxNumStepps"] == 500 and opts["numChunks"] == 32 and opts["CUDABlockSize"] == 128
    assert opts["batchPercent"] == 1 and opts["sort"] is True and opts["offsetAccess"] is False
    assert opts["base_calcSAH"] is False and opts["base_doSync"] is False
    assert cfg["baseConfig"]["name"] == "BVHTest default run"


def test_host_commands_roundtrip(tmp_path, orc):
    vert, faces = scenes.uniform_soup(3000, seed=4)
    meshio.write_mesh_v3(tmp_path / "scene", vert, faces)
    nodes, _, _ = orc.lbvh_build(vert, faces)
    depth = orc.fix_levels(nodes)
    meshio.write_bvh_v9(tmp_path / "scene", nodes, name="in", tree_height=depth)
    cfg = _config(tmp_path, [{"cmd": "load"}, {"cmd": "BVHImport", "options": {"name": "in"}}, {"cmd": "validate"},
                             {"cmd": "BVHExport", "options": {"name": "out"}}, {"cmd": "status"},
                             {"cmd": "writeData", "options": {"outFile": "%d/%i/stats_%n.json"}}])
    assert _run(cfg) == 0
    out, meta = meshio.read_bvh_v9(tmp_path / "scene", "out")
    assert np.array_equal(out.view(np.uint8), nodes.view(np.uint8)) and meta["treeHeight"] == depth
    stats = json.loads((tmp_path / "scene" / "stats_t.json").read_text())
    assert stats["numFaces"] == 3000 and stats["numBVHNodes"] == 5999 and stats["numVert"] == 9000
    # the config file was rewritten with every default filled in (src/main.cpp:166-169)
    rewritten = json.loads(cfg.read_text())
    assert rewritten["commands"][1]["options"] == {"name": "in"}


def test_validate_reports_a_broken_tree(tmp_path, orc):
    vert, faces = scenes.uniform_soup(500, seed=5)
    meshio.write_mesh_v3(tmp_path / "scene", vert, faces)
    nodes, _, _ = orc.lbvh_build(vert, faces)
    orc.fix_levels(nodes)
    nodes[7]["parent"] = 3  # plant a wrong parent link
    meshio.write_bvh_v9(tmp_path / "scene", nodes, name="bad", tree_height=int(nodes["level"].max()))
    cfg = _config(tmp_path, [{"cmd": "load"}, {"cmd": "BVHImport", "options": {"name": "bad"}}, {"cmd": "validate"},
                             {"cmd": "writeData"}])
    # validate returns WARNING, which does not stop the input: writeData still runs
    assert _run(cfg) == 0
    assert (tmp_path / "scene" / "rData_t.json").exists()


def test_errors_stop_an_input(tmp_path):
    cfg = _config(tmp_path, [{"cmd": "load"}, {"cmd": "writeData"}])  # no data.json: IO_ERROR
    assert _run(cfg) == 2
    assert not (tmp_path / "scene" / "rData_t.json").exists()


@pytest.mark.gpu
def test_gpu_pipeline_matches_oracle(tmp_path, orc):
    n = 20000
    vert, faces = scenes.uniform_soup(n, seed=6)
    meshio.write_mesh_v3(tmp_path / "scene", vert, faces)
    cam = dict(scenes.camera_default(), width=96, height=64)
    meshio.write_cameras_v1(tmp_path / "scene", [cam])
    cfg = _config(tmp_path, [
        {"cmd": "load"}, {"cmd": "camImport"}, {"cmd": "copyToGPU"},
        {"cmd": "LBVH"},
        {"cmd": "bittner13GPU", "options": {"maxNumStepps": 4, "base_calcSAH": True}},
        {"cmd": "CUDATracer"},
        {"cmd": "copyToHost", "options": {"fixLevels": True}},
        {"cmd": "validate"}, {"cmd": "BVHExport"}, {"cmd": "writeData"}, {"cmd": "writeImg"}])
    assert _run(cfg) == 0
    got, meta = meshio.read_bvh_v9(tmp_path / "scene")
    start, _, _ = orc.lbvh_build(vert, faces)
    ref, trace, _ = orc.bittner_chunked(start, 4)
    depth = orc.fix_levels(ref)
    assert np.array_equal(got.view(np.uint8), ref.view(np.uint8))
    assert meta["treeHeight"] == depth
    stats = json.loads((tmp_path / "scene" / "rData_t.json").read_text())
    sahs = [s["sah"] for s in stats["optStepps"]]
    assert len(sahs) == 5 and np.allclose(sahs, trace, rtol=1e-6)
    assert stats["numTotal"] == 4 * (int(np.float32(0.01) * np.float32(2 * n - 1)) // 32) * 32
    assert (tmp_path / "t_CUDA_cam_0.ppm").stat().st_size > 96 * 64 * 3


@pytest.mark.gpu
def test_learned_scorer_option(tmp_path, gpu):
    """bittner13GPU{learnedScorer} selects with the scorer read from the file: same tree as the API."""
    import torch
    n = 12000
    vert, faces = scenes.uniform_soup(n, seed=21)
    meshio.write_mesh_v3(tmp_path / "scene", vert, faces)
    m = gpu.Mlp(seed=11)
    m.save(tmp_path / "scorer.f32")
    cfg = _config(tmp_path, [
        {"cmd": "load"}, {"cmd": "copyToGPU"}, {"cmd": "LBVH"},
        {"cmd": "bittner13GPU", "options": {"maxNumStepps": 3, "learnedScorer": "scorer.f32"}},
        {"cmd": "copyToHost", "options": {"fixLevels": False}}, {"cmd": "BVHExport"}])
    assert _run(cfg) == 0
    got, _ = meshio.read_bvh_v9(tmp_path / "scene")
    v = torch.from_numpy(vert).cuda()
    f = torch.from_numpy(faces.view(np.int32)).cuda()
    nodes = gpu.LBVH(n).build(v, f)
    opt = gpu.Bittner13GPU(nodes)
    opt.set_scorer(gpu.Mlp.load(tmp_path / "scorer.f32"))
    opt.run(3)
    want = gpu.nodes_to_numpy(nodes)
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    cfg2 = _config(tmp_path, [{"cmd": "load"}, {"cmd": "copyToGPU"}, {"cmd": "LBVH"},
                              {"cmd": "bittner13GPU", "options": {"maxNumStepps": 1, "learnedScorer": "missing.f32"}}])
    assert _run(cfg2) == 2  # IO_ERROR stops the input


def test_malformed_configs_report_errors_without_crashing(tmp_path):
    """Bad JSON, a missing config file or input mesh give an error status; an unknown command is
    skipped with a warning; wrongly typed sections run nothing. None of them crashes the process."""
    cases = {
        "bad": ("{ not json", lambda r: r != 0),
        "missing_input": (json.dumps({"baseConfig": {"name": "x", "basePath": str(tmp_path), "input": ["nope"]},
                                      "commands": [{"cmd": "load"}]}), lambda r: r == 2),
        "unknown": (json.dumps({"baseConfig": {"name": "x", "basePath": str(tmp_path), "input": []},
                                "commands": [{"cmd": "frobnicate"}]}), lambda r: r == 0),
        "types": (json.dumps({"baseConfig": {"name": 5, "basePath": 7, "input": "scene"},
                              "commands": {"cmd": "load"}}), lambda r: r == 0),
        "array": ("[]", lambda r: r == 0),
    }
    for name, (text, ok) in cases.items():
        p = tmp_path / f"{name}.json"
        p.write_text(text)
        r = _run(p)
        assert ok(r), (name, r)
    assert _run(tmp_path / "no_such_config.json") != 0
