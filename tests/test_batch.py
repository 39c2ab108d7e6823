"""Batched frames: many independent frames of uneven size in one captured
kernel chain (include/rsrgpu.h rsrgpu_batch_*).

Bars:
  * every frame of a batch equals the same frame rendered alone through
    rsrgpu_run() with the same tiling: colour and depth bit-exact, canonical
    tile streams bit-exact
  * small frames also equal the oracle (colour with gamma off, depth)
  * graph replays read the inputs as they are at replay time
  * a frame whose tile-list pool is too small is regrown and re-run
  * the autotuner returns valid tilings and capacities that hold the frame
"""
import numpy as np
import pytest

from rsr_gb300 import scenes


def test_batch_generator_shape():
    fr = scenes.batch_frames(seed=0, nframes=64, tris=(1_000, 1_000_000))
    assert len(fr) == 64
    counts = np.array([f.ntris for f in fr])
    assert counts.min() >= 1_000 and counts.max() <= 1_000_000
    # log-uniform: about half the frames below the geometric mean (31 623)
    assert 20 <= (counts < 31_623).sum() <= 44
    sizes = {(f.width, f.height) for f in fr}
    assert sizes <= set(scenes.BATCH_RESOLUTIONS) and len(sizes) >= 4
    again = scenes.batch_frames(seed=0, nframes=64, tris=(1_000, 1_000_000))
    assert [f.ntris for f in again] == list(counts) and [(f.width, f.height) for f in again] == [(f.width, f.height) for f in fr]


def test_multi_draw_plain_frame_matches_reference(built):
    """plain_raster above 10 922 triangles splits into several draws; the
    oracle renders such a frame exactly as rsr does (x86 hosts with the
    reference built)."""
    import oracle
    if not oracle.ref_available():
        pytest.skip("reference library not built on this host")
    sc = scenes.plain_raster(seed=3, ntris=25_000, width=320, height=180, tile_blocks=(2, 2))
    outs = []
    for which in ("ref", "oracle"):
        c, d = oracle.CpuRenderer(which).render(sc, False)
        outs.append((c, d.view(np.uint32)))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


# ---------------------------------------------------------------- GPU
TILINGS = [(8, 8), (16, 16), (16, 8), (32, 32), (32, 16), (64, 32)]


def _device_frame(sc):
    import torch
    dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
    col = torch.zeros(sc.width * sc.height, dtype=torch.int32, device="cuda")
    dep = torch.zeros(sc.width * sc.height, dtype=torch.float32, device="cuda")
    gl = sc.record(ref=dev.__getitem__, color=col, depth=dep, gamma=False)
    return dev, col, dep, gl


def _single(gpu, sc, tile):
    """The frame alone through rsrgpu_run with tile edge `tile`."""
    import torch
    dev, col, dep, gl = _device_frame(sc)
    gpu.Reset(sc.width, sc.height, (tile // 8, tile // 8))
    gpu.Run(gl)
    gpu.Wait()
    torch.cuda.synchronize()
    return col.cpu().numpy().view(np.uint32), dep.cpu().numpy().view(np.uint32), gpu.tiles()


@pytest.fixture(scope="module")
def gpu(built):
    from rsr_gb300.gpu import GPU
    g = GPU(0)
    g.InstallDefaults()
    yield g
    g.close()


@pytest.fixture(scope="module")
def batch(built):
    from rsr_gb300.gpu import Batch
    b = Batch(0)
    b.InstallDefaults()
    yield b
    b.close()


def _small_batch(seed, n):
    return scenes.batch_frames(seed=seed, nframes=n, tris=(1_000, 60_000),
                               resolutions=((320, 180), (640, 360), (1280, 720), (1920, 1080)))


@pytest.mark.gpu
def test_batch_equals_single_frames(gpu, batch):
    import torch
    frames = _small_batch(1, 12)
    made = [_device_frame(sc) for sc in frames]
    descs = []
    for i, (sc, (dev, col, dep, gl)) in enumerate(zip(frames, made)):
        tile, region = TILINGS[i % len(TILINGS)]
        descs.append((gl, sc.width, sc.height, tile, region, 0))
    batch.submit(descs)
    batch.run()
    batch.wait()
    torch.cuda.synchronize()
    for i, (sc, (dev, col, dep, gl)) in enumerate(zip(frames, made)):
        tile = descs[i][3]
        bc, bd = col.cpu().numpy().view(np.uint32), dep.cpu().numpy().view(np.uint32)
        btiles = batch.frame(i).tiles()
        sc_col, sc_dep, stiles = _single(gpu, sc, tile)
        assert np.array_equal(bd, sc_dep), "frame %d: depth differs" % i
        assert np.array_equal(bc, sc_col), "frame %d: colour differs" % i
        assert btiles == stiles, "frame %d: tile streams differ" % i
    assert batch.last_ms() > 0


@pytest.mark.gpu
def test_batch_matches_oracle(batch):
    import oracle
    import torch
    cpu = oracle.CpuRenderer("oracle")
    frames = [scenes.plain_raster(seed=50 + i, ntris=n, width=w, height=h, tile_blocks=(t // 8, t // 8))
              for i, (n, w, h, t) in enumerate([(3000, 320, 180, 8), (12000, 640, 360, 16), (25000, 640, 360, 32)])]
    made = [_device_frame(sc) for sc in frames]
    batch.submit([(m[3], sc.width, sc.height, sc.tile_blocks[0] * 8, 0, 0) for sc, m in zip(frames, made)])
    batch.run()
    batch.wait()
    torch.cuda.synchronize()
    for i, (sc, (dev, col, dep, gl)) in enumerate(zip(frames, made)):
        oc, od = cpu.render(sc, False)
        assert np.array_equal(dep.cpu().numpy().view(np.uint32), od.view(np.uint32)), i
        assert np.array_equal(col.cpu().numpy().view(np.uint32), oc), i
        assert batch.frame(i).tiles() == cpu.tiles(), i


@pytest.mark.gpu
def test_graph_replay_reads_current_inputs(batch):
    import torch
    frames = _small_batch(2, 5)
    made = [_device_frame(sc) for sc in frames]
    batch.submit([(m[3], sc.width, sc.height, 16, 0, 0) for sc, m in zip(frames, made)])
    batch.run()
    batch.wait()
    first = [m[1].clone() for m in made]
    batch.run()
    batch.wait()
    assert all(torch.equal(a, m[1]) for a, m in zip(first, made))
    # move frame 0's triangles: the replay renders the new positions
    made[0][0]["px"].mul_(0.5)
    batch.run()
    batch.wait()
    torch.cuda.synchronize()
    assert not torch.equal(first[0], made[0][1])
    assert all(torch.equal(first[i], made[i][1]) for i in range(1, len(made)))


@pytest.mark.gpu
def test_batch_regrows_a_small_tile_pool(gpu, batch):
    import torch
    frames = _small_batch(3, 4)
    made = [_device_frame(sc) for sc in frames]
    batch.submit([(m[3], sc.width, sc.height, 16, 0, 1024) for sc, m in zip(frames, made)])
    batch.run()
    batch.wait()
    torch.cuda.synchronize()
    for sc, (dev, col, dep, gl) in zip(frames, made):
        c, d, _ = _single(gpu, sc, 16)
        assert np.array_equal(col.cpu().numpy().view(np.uint32), c)
        assert np.array_equal(dep.cpu().numpy().view(np.uint32), d)


@pytest.mark.gpu
def test_autotuner_choices(batch):
    import torch
    frames = _small_batch(4, 6)
    made = [_device_frame(sc) for sc in frames]
    choice = batch.tune([(m[3], sc.width, sc.height) for sc, m in zip(frames, made)], reps=2)
    assert len(choice) == len(frames)
    for tile, region, cap in choice:
        assert tile in (8, 16, 32, 64) and region in (8, 16, 32) and region <= tile
        assert cap >= 1024
    batch.submit([(m[3], sc.width, sc.height, t, r, c) for (sc, m), (t, r, c) in zip(zip(frames, made), choice)])
    batch.run()
    batch.wait()
    torch.cuda.synchronize()
    for i in range(len(frames)):
        fc = batch.frame(i)
        fc.tiles()   # fills the frame's tile-list statistics
        st = fc.stats()
        # the tuned capacity held the frame (no regrowth needed): entries fit
        assert st["total_tile_records"] + st["total_clipped_records"] <= choice[i][2]
