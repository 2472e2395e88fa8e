"""The autotuner's cache file format (CPU) and its choices (GPU): tuning chooses launch shapes only,
so a tuned model's substeps must be bit-identical to an untuned model's."""
from __future__ import annotations

import numpy as np
import pytest

import vkfluidsim_gb300 as vfs
from vkfluidsim_gb300 import workloads as W


def test_tune_cache_file_round_trip(tmp_path):
    vfs.tune_cache_clear()
    f = tmp_path / "tune.txt"
    # A full line, and a line without the force shape (which then follows the neighbour shape).
    f.write_text("# header\nsm103_152sms_n32768_s1_00000000000000aa 7 12 96 8 512 128 8\n"
                 "sm103_152sms_n65536_s1_00000000000000bb 8 16 64 12 256\n")
    vfs.tune_cache_load(str(f))
    out = tmp_path / "out.txt"
    vfs.tune_cache_save(str(out))
    lines = [ln for ln in out.read_text().splitlines() if not ln.startswith("#")]
    assert lines == ["sm103_152sms_n32768_s1_00000000000000aa 7 12 96 8 512 128 8 0",
                     "sm103_152sms_n65536_s1_00000000000000bb 8 16 64 12 256 64 12 0"]
    # A line with the walk-staging value keeps it.
    f.write_text("sm103_152sms_n9_s1_00000000000000cc 8 16 128 8 256 128 8 1\n")
    vfs.tune_cache_load(str(f))
    vfs.tune_cache_save(str(out))
    assert "sm103_152sms_n9_s1_00000000000000cc 8 16 128 8 256 128 8 1" in out.read_text()
    vfs.tune_cache_clear()


@pytest.mark.parametrize("bad", ["key 7 12 100 3 512\n", "key 9 12 128 6 256\n", "key 7\n",
                                 "key 7 12 128 6 256 100 3\n", "key 7 12 128 6 256 128\n",
                                 "key 7 12 128 6 256 128 6 2\n"])
def test_tune_cache_rejects_bad_lines(tmp_path, bad):
    f = tmp_path / "bad.txt"
    f.write_text(bad)
    with pytest.raises(vfs.VfsError) as e:
        vfs.tune_cache_load(str(f))
    assert e.value.code == 5  # VFS_ERR_PARSE


def test_tune_cache_missing_file_is_an_io_error(tmp_path):
    with pytest.raises(vfs.VfsError) as e:
        vfs.tune_cache_load(str(tmp_path / "absent.txt"))
    assert e.value.code == 4  # VFS_ERR_IO


def _state(m):
    s = m.copy_data_buffers()
    ids = m.get_ids()
    x = np.empty_like(s["positions"])
    v = np.empty_like(s["velocities"])
    x[ids] = s["positions"]
    v[ids] = s["velocities"]
    return x, v


@pytest.mark.gpu
# The models below have 110,592 particles: large enough for one lane per particle in the density
# pass, where its launch shapes apply (smaller models run it three lanes per particle with one
# fixed shape).
def test_autotuned_model_is_bit_identical_to_default():
    vfs.tune_cache_clear()
    w = W.dam_break(dims=(48, 48, 48), map_res=32, seed=2)
    ref = W.build_model(w)
    ref.substeps(4)
    m = W.build_model(w)
    chosen = m.autotune(repeats=2, use_cache=False)
    assert chosen == m.get_tune_config()
    m.substeps(4)
    x0, v0 = _state(ref)
    x1, v1 = _state(m)
    assert np.array_equal(x0, x1) and np.array_equal(v0, v1)
    k0, p0, o0 = ref.get_neighbor_arrays()
    k1, p1, o1 = m.get_neighbor_arrays()
    assert np.array_equal(k0, k1) and np.array_equal(p0, p1) and np.array_equal(o0, o1)
    # A second model of the same workload takes the cached choice.
    m2 = W.build_model(w)
    assert m2.autotune(repeats=2, use_cache=True) == chosen


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(128, 6), (128, 8), (96, 8), (64, 12)])
@pytest.mark.parametrize("cell_block", [128, 512])
def test_every_launch_shape_gives_the_same_step(shape, cell_block):
    w = W.dam_break(dims=(48, 48, 48), map_res=24, seed=5)
    ref = W.build_model(w)
    ref.substeps(3)
    m = W.build_model(w)
    m.set_tune_config(nbr_block=shape[0], nbr_min_blocks=shape[1], cell_block=cell_block,
                      sort_digit_bits=6, sort_tile_items=8, force_block=shape[0],
                      force_min_blocks=shape[1])
    m.substeps(3)
    x0, v0 = _state(ref)
    x1, v1 = _state(m)
    assert np.array_equal(x0, x1) and np.array_equal(v0, v1)


@pytest.mark.gpu
def test_force_shape_apart_from_density_shape():
    w = W.dam_break(dims=(48, 48, 48), map_res=24, seed=6)
    ref = W.build_model(w)
    ref.substeps(3)
    m = W.build_model(w)
    m.set_tune_config(nbr_block=64, nbr_min_blocks=12, force_block=128, force_min_blocks=6)
    assert m.get_tune_config()["force_block"] == 128
    m.substeps(3)
    x0, v0 = _state(ref)
    x1, v1 = _state(m)
    assert np.array_equal(x0, x1) and np.array_equal(v0, v1)
    # 0 x 0 selects the neighbour passes' shape.
    m.set_tune_config(nbr_block=64, nbr_min_blocks=12, force_block=0, force_min_blocks=0)
    cfg = m.get_tune_config()
    assert (cfg["force_block"], cfg["force_min_blocks"]) == (64, 12)


@pytest.mark.gpu
def test_invalid_tune_config_is_rejected():
    m = W.build_model(W.dam_break(dims=(8, 8, 8), map_res=0))
    with pytest.raises(vfs.VfsError):
        m.set_tune_config(nbr_block=100)
    with pytest.raises(vfs.VfsError):
        m.set_tune_config(force_block=100)
    with pytest.raises(vfs.VfsError):
        m.set_tune_config(cell_block=1000)


@pytest.mark.gpu
def test_batch_autotune_keeps_results():
    scenes = W.batched_scenes(n_scenes=6, n_min=2048, n_max=8192, map_res=16, seed=9)
    a = W.build_batch(scenes)
    a.substeps(2)
    b = W.build_batch(scenes)
    b.autotune(repeats=1, use_cache=False)
    b.substeps(2)
    for s in range(len(scenes)):
        sa, sb = a.copy_data_buffers(s), b.copy_data_buffers(s)
        assert np.array_equal(sa["positions"][np.argsort(a.get_ids(s))],
                              sb["positions"][np.argsort(b.get_ids(s))])
