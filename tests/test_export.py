"""Headless state export: snapshot files (CPU: the reader on a hand-made file; GPU: export, import
and the overlapped recorder against copy_data_buffers)."""
from __future__ import annotations

import json

import numpy as np
import pytest

import vkfluidsim_gb300 as vfs
from vkfluidsim_gb300 import workloads as W


def _write_snapshot(prefix, pos, vel, dens, substeps=0):
    n = len(dens)
    (prefix.parent / (prefix.name + ".bin")).write_bytes(
        pos.astype("<f4").tobytes() + vel.astype("<f4").tobytes() + dens.astype("<f4").tobytes())
    meta = {"format": "vkfluidsim_gb300.state", "version": 1, "binary": prefix.name + ".bin",
            "particles": n, "order": "particle id", "substeps": substeps, "time": 0.0,
            "arrays": {"positions": {"dtype": "<f4", "shape": [n, 3], "offset": 0},
                       "velocities": {"dtype": "<f4", "shape": [n, 3], "offset": 12 * n},
                       "densities": {"dtype": "<f4", "shape": [n], "offset": 24 * n}},
            "parameters": {}}
    (prefix.parent / (prefix.name + ".json")).write_text(json.dumps(meta))


def test_reader_parses_the_documented_layout(tmp_path):
    rng = np.random.default_rng(0)
    pos, vel, dens = rng.random((5, 3)), rng.random((5, 3)), rng.random(5)
    _write_snapshot(tmp_path / "s", pos, vel, dens, substeps=7)
    s = vfs.read_state(tmp_path / "s")
    assert s["substeps"] == 7 and s["particles"] == 5
    assert np.array_equal(s["positions"], pos.astype(np.float32))
    assert np.array_equal(s["velocities"], vel.astype(np.float32))
    assert np.array_equal(s["densities"], dens.astype(np.float32))


def test_reader_rejects_other_formats(tmp_path):
    (tmp_path / "x.json").write_text(json.dumps({"format": "other", "version": 1}))
    with pytest.raises(ValueError):
        vfs.read_state(tmp_path / "x")


def _by_id(m):
    s = m.copy_data_buffers()
    ids = m.get_ids()
    out = {}
    for k in ("positions", "velocities", "densities"):
        a = np.empty_like(s[k])
        a[ids] = s[k]
        out[k] = a
    return out


@pytest.mark.gpu
def test_export_matches_copy_data_buffers(tmp_path):
    w = W.dam_break(dims=(16, 16, 16), map_res=16, seed=4)
    m = W.build_model(w)
    m.substeps(3)
    m.export_state(tmp_path / "snap")
    s = vfs.read_state(tmp_path / "snap")
    ref = _by_id(m)
    assert s["substeps"] == 3
    for k in ("positions", "velocities", "densities"):
        assert np.array_equal(s[k], ref[k]), k
    assert s["parameters"]["smooth_radius"] == pytest.approx(w.sim.smooth_radius)


@pytest.mark.gpu
def test_import_restores_the_state(tmp_path):
    w = W.dam_break(dims=(16, 16, 16), map_res=16, seed=4)
    m = W.build_model(w)
    m.substeps(2)
    m.export_state(tmp_path / "snap")
    m2 = W.build_model(w)
    m2.import_state(tmp_path / "snap")
    a, b = _by_id(m), _by_id(m2)
    assert np.array_equal(a["positions"], b["positions"])
    assert np.array_equal(a["velocities"], b["velocities"])
    m.substeps(2)
    m2.substeps(2)
    a, b = _by_id(m), _by_id(m2)
    # Same state, particles in another order within their buckets: sums differ by rounding only.
    scale = np.abs(a["positions"]).max()
    assert np.abs(a["positions"] - b["positions"]).max() <= 1e-5 * scale


@pytest.mark.gpu
def test_import_rejects_a_size_mismatch(tmp_path):
    m = W.build_model(W.dam_break(dims=(8, 8, 8), map_res=0))
    m.export_state(tmp_path / "snap")
    m2 = W.build_model(W.dam_break(dims=(8, 8, 9), map_res=0))
    with pytest.raises(vfs.VfsError):
        m2.import_state(tmp_path / "snap")


@pytest.mark.gpu
def test_recorder_frames_equal_plain_stepping(tmp_path):
    w = W.dam_break(dims=(16, 16, 16), map_res=16, seed=6)
    m = W.build_model(w)
    m.record(7, 2, tmp_path / "rec")
    ref = W.build_model(w)
    for f in range(3):
        ref.substeps(2)
        s = vfs.read_state(tmp_path / f"rec_f{f:06d}")
        r = _by_id(ref)
        assert s["substeps"] == 2 * (f + 1)
        assert np.array_equal(s["positions"], r["positions"])
        assert np.array_equal(s["velocities"], r["velocities"])
    assert not (tmp_path / "rec_f000003.json").exists()
    ref.substeps(1)
    assert np.array_equal(_by_id(m)["positions"], _by_id(ref)["positions"])


@pytest.mark.gpu
def test_batch_recorder_writes_every_scene(tmp_path):
    scenes = W.batched_scenes(n_scenes=3, n_min=2048, n_max=4096, map_res=0, seed=2)
    b = W.build_batch(scenes)
    b.record(4, 2, tmp_path / "b")
    for s, w in enumerate(scenes):
        for f in range(2):
            snap = vfs.read_state(tmp_path / f"b_s{s}_f{f:06d}")
            assert snap["positions"].shape == (w.n, 3)
    last = vfs.read_state(tmp_path / "b_s1_f000001")
    st = b.copy_data_buffers(1)
    pos = np.empty_like(st["positions"])
    pos[b.get_ids(1)] = st["positions"]
    assert np.array_equal(last["positions"], pos)
