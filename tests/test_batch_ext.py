"""Batches of the frames rsr's tile interpreter renders beyond plain draws:
float colour stores (rglv_gpu.cxx:345-383), instanced draws with ManyProgram
(CMD_DRAW_*_INSTANCED, rglv_gpu_impl.hxx:488-494) and OBJ1Program draws, in
one batch with plain frames.  rsr's loop renders any such frame
(rglv_gpu.cxx:119-432); a batch must give every frame the oracle's output:
depth, linear colour and float outputs bit-exact, tile streams equal.
"""
import numpy as np
import pytest

from rsr_gb300 import scenes


@pytest.fixture(scope="module")
def orc(built):
    import oracle
    return oracle.CpuRenderer("oracle")


@pytest.mark.gpu
def test_batch_of_float_store_instanced_obj1_and_plain_frames(built, orc):
    import torch
    from rsr_gb300.gpu import Batch
    plain = scenes.plain_raster(seed=5, ntris=3000, width=320, height=180, tile_blocks=(4, 4), spread=0.4)
    fstore = scenes.float_store_frame(seed=23, ntris=2000, width=320, height=180)
    fmid = scenes.float_store_frame(seed=24, ntris=2000, width=192, height=128, color_depth=True, mid=True)
    inst = scenes.instanced_scene(seed=45, ninst=600, width=320, height=180)
    obj1 = scenes.obj1_scene(seed=55, nspheres=10, width=320, height=180)

    # the oracle's outputs
    want = {}
    for sc in (plain, inst, obj1):
        oc, od = orc.render(sc, False)
        want[sc.name] = {"color": oc.copy(), "depth": od.copy(), "tiles": orc.tiles()}
    for sc in (fstore, fmid):
        for v in sc.outputs.values():
            v[:] = 0
        orc.render_gl(sc.record(gamma=False), sc.width, sc.height, sc.tile_blocks)
        want[sc.name] = {k: v.copy() for k, v in sc.outputs.items()}
        want[sc.name]["tiles"] = orc.tiles()

    # one batch of all five, device inputs and outputs
    frames, keep = [], []
    for sc in (plain, inst, obj1):
        dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
        col = torch.zeros(sc.width * sc.height, dtype=torch.int32, device="cuda")
        dep = torch.zeros(sc.width * sc.height, dtype=torch.float32, device="cuda")
        keep.append((sc, dev, {"color": col, "depth": dep}))
        frames.append((sc.record(ref=dev.__getitem__, color=col, depth=dep, gamma=False), sc.width, sc.height, 32, 0, 0))
    for sc in (fstore, fmid):
        dev = {k: torch.from_numpy(v).cuda() for k, v in sc.arrays.items()}
        out = {k: torch.zeros(v.size, dtype=torch.float32 if v.dtype == np.float32 else torch.int32, device="cuda")
               for k, v in sc.outputs.items()}
        keep.append((sc, dev, out))
        frames.append((sc.record(ref=dev.__getitem__, outputs=out, gamma=False), sc.width, sc.height, 32, 0, 0))
    b = Batch(0)
    try:
        b.InstallDefaults()
        b.submit(frames)
        for _ in range(2):   # a replay renders the same frames again
            for _, _, out in keep:
                for t in out.values():
                    t.zero_()
            b.run()
            b.wait()
            torch.cuda.synchronize()
            for i, (sc, _, out) in enumerate(keep):
                w = want[sc.name]
                for k, t in out.items():
                    got = t.cpu().numpy().view(np.uint32)
                    exp = np.ascontiguousarray(w[k]).view(np.uint32)
                    assert np.array_equal(got, exp), "%s: %s differs from the oracle" % (sc.name, k)
                assert b.frame(i).tiles() == w["tiles"], "%s: tile streams differ" % sc.name
    finally:
        b.close()
