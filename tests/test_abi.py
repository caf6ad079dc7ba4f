"""The C ABI without a GPU: the library loads, exports every function the
header declares, its struct layouts match the ctypes view, the host-side
BVH check agrees with the oracle, and argument errors come back as statuses."""
import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import trayracer_gb300 as tr
from oracle import Oracle
from trayracer_gb300 import _abi
from trayracer_gb300.renderer import SceneDescHolder
from trayracer_gb300.scenes import random_soup

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "trayracer.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:tr_status|const char\*)\s+(tr_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_function():
    lib = _abi.load_library()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(_abi.FUNCTIONS), "ctypes table out of sync with the header"


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc missing")
def test_struct_layouts_match_ctypes(tmp_path):
    structs = {
        "tr_kernel_settings": _abi.KernelSettings,
        "tr_camera": _abi.Camera,
        "tr_material_desc": _abi.MaterialDesc,
        "tr_mesh_desc": _abi.MeshDesc,
        "tr_scene_desc": _abi.SceneDesc,
        "tr_config": _abi.Config,
        "tr_statistics": _abi.Statistics,
        "tr_scene_info": _abi.SceneInfo,
        "tr_buffers": _abi.Buffers,
        "tr_instance_desc": _abi.InstanceDesc,
        "tr_tuning": _abi.Tuning,
        "tr_tune_report": _abi.TuneReport,
        "tr_batch_item": _abi.BatchItem,
        "tr_batch_info": _abi.BatchInfo,
        "tr_batch_statistics": _abi.BatchStatistics,
        "tr_ray_pick_result": _abi.RayPickResult,
        "tr_sky_desc": _abi.SkyDesc,
        "tr_texture_desc": _abi.TextureDesc,
        "tr_scene_file_info": _abi.SceneFileInfo,
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-o", str(exe), str(src)], check=True)
    out = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                              check=True).stdout.split("\n") if line)
    for cname, py in structs.items():
        assert int(out[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(out[f"{cname}.{f}"]) == getattr(py, f).offset, f"{cname}.{f}"


def test_status_strings():
    lib = _abi.load_library()
    assert lib.tr_status_string(0) == b"ok"
    assert lib.tr_status_string(7) == b"device fault"


def test_null_arguments_are_rejected():
    lib = _abi.load_library()
    assert lib.tr_create(None, None) == 1
    assert lib.tr_destroy(None) == 1
    assert lib.tr_trace_host(None, None, None, 0, 0.0, 0, None, None) == 1


def _rays(scene, n, seed):
    rng = np.random.default_rng(seed)
    lo, hi = scene.positions.min(0), scene.positions.max(0)
    O = np.zeros((n, 4), np.float32)
    D = np.zeros((n, 4), np.float32)
    O[:, :3] = rng.uniform(lo - 0.2 * (hi - lo), hi + 0.2 * (hi - lo), (n, 3))
    d = rng.normal(size=(n, 3))
    D[:, :3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    return O, D


def _host_trace(scene, O, D, any_hit=False, leaf=0, tmin=1e-3, quant=False):
    lib = _abi.load_library()
    h = SceneDescHolder(scene, leaf_size=leaf)
    n = O.shape[0]
    hits = np.zeros((n, 4), np.uint32)
    counts = np.zeros((n, 2), np.uint32)
    flags = int(any_hit) | (2 if quant else 0)  # bit 1: 8-bit quantized child boxes
    st = lib.tr_trace_host(C.byref(h.desc), O.ctypes.data, D.ctypes.data, n, tmin, flags, hits.ctypes.data,
                           counts.ctypes.data)
    assert st == 0
    return hits, counts


def _check_closest(scene, O, D, hits):
    o = Oracle(scene)
    want = o.trace_closest(O, D, 1e-3)
    same = (hits == want).all(axis=1)
    for i in np.where(~same)[0]:
        # a different primitive is only allowed on a near tie (|dt| <= 1e-6 t)
        t_got = float(hits[i, 3].view(np.float32))
        t_want = float(want[i, 3].view(np.float32))
        assert abs(t_got - t_want) <= 1e-6 * abs(t_want), (i, hits[i], want[i])
        ties = o.ties(O[i], D[i], 1e-3, t_want, with_instances=True)
        assert (int(hits[i, 1]), int(hits[i, 2])) in ties, (i, hits[i], ties)
    return same.mean()


@pytest.mark.parametrize("quant", [False, True], ids=["fp32", "quantized"])
@pytest.mark.parametrize("leaf", [1, 2, 3])
def test_host_cwbvh_closest_hit_matches_oracle(leaf, quant):
    scene = random_soup(4000, seed=leaf)
    O, D = _rays(scene, 8000, seed=leaf)
    hits, counts = _host_trace(scene, O, D, leaf=leaf, quant=quant)
    assert _check_closest(scene, O, D, hits) == 1.0
    assert counts[:, 0].min() >= 1


@pytest.mark.parametrize("quant", [False, True], ids=["fp32", "quantized"])
def test_host_cwbvh_cornell_and_heightfield(quant):
    for scene in (tr.cornell_box(), tr.heightfield(n=96, width=8, height=8)):
        O, D = _rays(scene, 6000, seed=3)
        hits, _ = _host_trace(scene, O, D, quant=quant)
        # coplanar faces (box bottoms on the floor) are the only ties
        assert _check_closest(scene, O, D, hits) > 0.99


def test_host_node_layouts_visit_counts():
    """Exact fp32 child boxes are never larger than their outward-rounded 8-bit
    quantization, so no ray visits more nodes with them."""
    scene = tr.heightfield(n=96, width=8, height=8)
    O, D = _rays(scene, 6000, seed=7)
    _, c32 = _host_trace(scene, O, D)
    _, c8 = _host_trace(scene, O, D, quant=True)
    assert (c32[:, 0] <= c8[:, 0]).all()
    assert c32[:, 0].sum() < c8[:, 0].sum()


@pytest.mark.parametrize("quant", [False, True], ids=["fp32", "quantized"])
def test_host_cwbvh_any_hit_matches_oracle(quant):
    scene = random_soup(3000, seed=9)
    O, D = _rays(scene, 6000, seed=4)
    D[:, 3] = np.random.default_rng(5).uniform(0.05, 2.0, 6000).astype(np.float32)
    hits, _ = _host_trace(scene, O, D, any_hit=True, quant=quant)
    occluded_host = hits[:, 2] != 0xFFFFFFFF
    L = D.copy()
    L[:, 3] = D[:, 3] + 2e-3  # orc_trace_any uses tmax = dist - 2 eps
    occ = Oracle(scene).trace_any(O, L, 1e-3).astype(bool)
    assert np.mean(occluded_host == occ) == 1.0


def test_host_cwbvh_empty_and_single_triangle():
    pos = np.array([[0, 0, 1], [1, 0, 1], [0, 1, 1]], np.float32)
    mats = np.array([tr.scenes.material()], tr.scenes.MATERIAL_DTYPE)
    one = tr.Scene("one", pos, None, None, np.array([[0, 1, 2]], np.uint32), np.zeros(1, np.uint32), mats)
    O = np.array([[0.2, 0.2, 0, 0], [2, 2, 0, 0]], np.float32)
    D = np.array([[0, 0, 1, 0], [0, 0, 1, 0]], np.float32)
    hits, _ = _host_trace(one, O, D)
    assert hits[0, 2] == 0 and abs(float(hits[0, 3].view(np.float32)) - 1.0) < 1e-6
    assert hits[1, 2] == 0xFFFFFFFF
    empty = tr.Scene("empty", np.zeros((0, 3), np.float32), None, None, np.zeros((0, 3), np.uint32),
                     np.zeros(0, np.uint32), mats)
    hits, _ = _host_trace(empty, O, D)
    assert np.all(hits[:, 2] == 0xFFFFFFFF)


def test_invalid_scene_rejected_by_host_entry():
    lib = _abi.load_library()
    scene = tr.cornell_box()
    bad = tr.Scene("bad", scene.positions, scene.normals, scene.texcoords, scene.indices.copy(),
                   scene.material_indices.copy(), scene.materials)
    bad.indices[0, 0] = 10 ** 6
    h = SceneDescHolder(bad)
    hits = np.zeros((1, 4), np.uint32)
    O = np.zeros((1, 4), np.float32)
    assert lib.tr_trace_host(C.byref(h.desc), O.ctypes.data, O.ctypes.data, 1, 1e-3, 0, hits.ctypes.data, None) == 1


def test_host_two_level_matches_oracle():
    """Instances: the instance BVH, then each mesh's BVH in object space (same ray
    transform and triangle test as the oracle), closest and any hit."""
    scene = tr.instanced_cornell()
    rng = np.random.default_rng(11)
    n = 12000
    O = np.zeros((n, 4), np.float32)
    D = np.zeros((n, 4), np.float32)
    O[:, :3] = rng.uniform(-0.95, 0.95, (n, 3))
    d = rng.normal(size=(n, 3))
    D[:, :3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    for leaf in (1, 3):
        hits, counts = _host_trace(scene, O, D, leaf=leaf)
        # the boxes' bottoms lie on the floor: coplanar ties are the only differences
        assert _check_closest(scene, O, D, hits) > 0.999
        assert counts[:, 0].min() >= 1
    inst = hits[hits[:, 2] != 0xFFFFFFFF, 1]
    assert set(np.unique(inst)) == set(range(len(scene.instances)))  # every instance is hit
    D[:, 3] = rng.uniform(0.05, 1.5, n).astype(np.float32)
    hits, _ = _host_trace(scene, O, D, any_hit=True)
    L = D.copy()
    L[:, 3] = D[:, 3] + 2e-3
    occ = Oracle(scene).trace_any(O, L, 1e-3).astype(bool)
    assert np.mean((hits[:, 2] != 0xFFFFFFFF) == occ) == 1.0


def test_two_level_scene_validation():
    scene = tr.instanced_cornell()
    scene.instances[3] = (17, scene.instances[3][1])  # a mesh that does not exist
    O = np.zeros((1, 4), np.float32)
    D = np.array([[0, 0, 1, 0]], np.float32)
    hits = np.zeros((1, 4), np.uint32)
    lib = _abi.load_library()
    h = SceneDescHolder(scene)
    assert lib.tr_trace_host(C.byref(h.desc), O.ctypes.data, D.ctypes.data, 1, 1e-3, 0, hits.ctypes.data, None) == 1
