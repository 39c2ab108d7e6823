"""Learned deferred shader: parameters, GPU training and serving.

The network (24 -> 64 -> 64 -> 64 -> 3, ReLU, BF16 weights and activations,
FP32 accumulation) maps the per-pixel features that rsrgpu_learned_features()
and the fused rsrgpu_shade_learned() compute from a G-buffer to the residual
sqrt(plain) - base, where plain is the linear RGB of the plain multi-light
shader and base the square root of the analytic virtual-light estimate from
the same features (the method without the network; the untrained network,
whose output layer is zero, reproduces it exactly).  All
arithmetic runs in this library's kernels: features and targets
(learned_features_kernel), forward + backward (mlp_train_kernel on tcgen05),
Adam (adam_kernel), inference with the per-tile gate and plain fallback
(shade_learned_kernel).  PyTorch only holds device memory.

Parameter layout (FP32 master copy, also the gradient layout): w1 [64][32] |
w2 [64][64] | w3 [64][64] | w4 [16][64] | b1 [64] | b2 [64] | b3 [64] | b4 [16]
(input columns 24..31 and output rows 3..15 zero).
"""
import json
import multiprocessing as mp
import os
import tempfile
import time

import numpy as np

from . import scenes
from .gpu import render_gbuffer

NWEIGHTS = 11264
NPARAMS = 11472
OFFSETS = {"w1": (0, (64, 32)), "w2": (2048, (64, 64)), "w3": (6144, (64, 64)), "w4": (10240, (16, 64)),
           "b1": (11264, (64,)), "b2": (11328, (64,)), "b3": (11392, (64,)), "b4": (11456, (16,))}
PSNR_40DB_MSE = 255.0 ** 2 / 1e4      # mean squared sRGB8 error of 40 dB
WEIGHTS_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "learned_shader.npz")


def init_params(seed=0):
    """He-initialised hidden layers, zero output layer (padding zero), FP32
    numpy vector."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS, np.float32)

    def put(name, value):
        off, shape = OFFSETS[name]
        p[off:off + int(np.prod(shape))] = np.asarray(value, np.float32).reshape(-1)

    w1 = np.zeros((64, 32)); w1[:, :24] = rng.standard_normal((64, 24)) * np.sqrt(2 / 24)
    put("w1", w1)
    put("w2", rng.standard_normal((64, 64)) * np.sqrt(2 / 64))
    put("w3", rng.standard_normal((64, 64)) * np.sqrt(2 / 64))
    # w4 and b4 start at zero: the untrained shader is exactly its analytic base
    return p


class LearnedShader:
    """Device-resident network: FP32 master parameters, Adam moments, and the
    BF16 weights / FP32 biases the kernels read."""

    def __init__(self, params=None, seed=0):
        import torch
        p = init_params(seed) if params is None else np.asarray(params, np.float32)
        assert p.shape == (NPARAMS,)
        self.params = torch.from_numpy(p.copy()).cuda()
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grad = torch.zeros_like(self.params)
        self.loss = torch.zeros(1, device="cuda")
        self.step = 0
        self.wbf = self.params[:NWEIGHTS].to(torch.bfloat16).contiguous()
        self.bias = self.params[NWEIGHTS:].clone()
        self.meta = {}

    def views(self):
        w, b = self.wbf, self.bias
        return {"w1": w[0:2048], "w2": w[2048:6144], "w3": w[6144:10240], "w4": w[10240:11264],
                "b1": b[0:64], "b2": b[64:128], "b3": b[128:192], "b4": b[192:208]}

    def numpy_params(self):
        return self.params.cpu().numpy().copy()

    def save(self, path, meta=None):
        os.makedirs(os.path.dirname(path), exist_ok=True)
        m = dict(self.meta, **(meta or {}))
        np.savez(path, params=self.numpy_params(), meta=np.frombuffer(json.dumps(m).encode(), np.uint8))

    @classmethod
    def load(cls, path=WEIGHTS_PATH):
        z = np.load(path)
        s = cls(params=z["params"])
        s.meta = json.loads(bytes(z["meta"]).decode()) if "meta" in z else {}
        return s

    def train_step(self, gpu, features, targets, index, lr):
        """One Adam step on the batch features[index] (tcgen05 forward + backward)."""
        self.step += 1
        gpu.mlp_grad(self.views(), features, targets, index, self.grad, self.loss)
        gpu.mlp_adam(self.params, self.grad, self.m, self.v, self.step, lr, self.wbf, self.bias)


# ---- training data ----
def _make_scene_file(args):
    """Worker: builds one deferred scene and saves its arrays (spawned process)."""
    seed, width, height, nobj, out = args
    sc = scenes.deferred_scene(seed=seed, width=width, height=height, nobj=nobj)
    np.savez(out, **sc.arrays)
    return out


def scene_files(seeds, width=1920, height=1080, nobj=2_000_000, workers=None, tmpdir=None):
    """Builds the deferred scenes of `seeds` in a spawned process pool (the
    scene generator is NumPy-bound) and yields (seed, npz path) in order."""
    tmpdir = tmpdir or tempfile.mkdtemp(prefix="rsrgpu_scenes_")
    jobs = [(s, width, height, nobj, os.path.join(tmpdir, "scene_%d.npz" % s)) for s in seeds]
    workers = workers or max(1, min(len(jobs), (os.cpu_count() or 2) // 2, 8))
    if workers == 1:
        for j in jobs:
            yield j[0], _make_scene_file(j)
        return
    # at most `workers` scene files wait on disk at a time (about 1.3 GB each at full size)
    with mp.get_context("spawn").Pool(workers) as pool:
        pending = [pool.apply_async(_make_scene_file, (j,)) for j in jobs[:workers]]
        for i, j in enumerate(jobs):
            path = pending[i].get()
            if i + workers < len(jobs):
                pending.append(pool.apply_async(_make_scene_file, (jobs[i + workers],)))
            yield j[0], path


class DeferredFrame:
    """G-buffer, camera and lights of one deferred scene on the device."""

    def __init__(self, gpu, seed, width=1920, height=1080, nobj=2_000_000, path=None):
        import torch
        if path is not None:
            z = np.load(path)
            sc = scenes.deferred_scene(seed=seed, width=width, height=height, nobj=nobj,
                                       arrays={k: z[k] for k in z.files})
        else:
            sc = scenes.deferred_scene(seed=seed, width=width, height=height, nobj=nobj)
        self.seed, self.width, self.height = seed, width, height
        # the vertex arrays stay on the device: the context keeps the submitted
        # G-buffer frame, and gpu.run() may render it again
        self.gbuf, self.dev = render_gbuffer(gpu, sc)
        self.lights = torch.from_numpy(np.ascontiguousarray(sc.lights, np.float32)).cuda()
        self.lights_np = np.ascontiguousarray(sc.lights, np.float32)
        self.ivp, self.eye = sc.ivp.copy(), sc.eye.copy()
        self.covered = (self.gbuf["albedo"] != 0)

    def features(self, gpu, targets=True):
        import torch
        n = self.width * self.height
        f = torch.zeros(n, 32, dtype=torch.bfloat16, device="cuda")
        t = torch.zeros(n, 3, dtype=torch.float32, device="cuda") if targets else None
        gpu.learned_features(self.gbuf, self.width, self.height, self.ivp, self.eye, self.lights, f, t)
        return f, t

    def shade_plain(self, gpu, out_srgb=None, out_linear=None, stream=None):
        gpu.shade_plain(self.gbuf, self.width, self.height, self.ivp, self.eye, self.lights,
                        out_srgb=out_srgb, out_linear=out_linear, stream=stream)

    def shade_learned(self, gpu, net, max_tile_mse=PSNR_40DB_MSE, out_srgb=None, out_linear=None,
                      tile_status=None, tile_mse=None, stream=None):
        gpu.shade_learned(net.views(), self.gbuf, self.width, self.height, self.ivp, self.eye, self.lights,
                          max_tile_mse=max_tile_mse, out_srgb=out_srgb, out_linear=out_linear,
                          tile_status=tile_status, tile_mse=tile_mse, stream=stream)

    @property
    def ntiles(self):
        return ((self.width + 31) // 32) * ((self.height + 31) // 32)


def collect_samples(gpu, seeds, per_seed, width=1920, height=1080, nobj=2_000_000, sample_seed=0, log=None):
    """Renders each seed's G-buffer on the GPU, builds features and targets on
    the GPU and keeps `per_seed` random covered pixels of each.  Returns
    device tensors (features bf16 [N][32], targets fp32 [N][3])."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(sample_seed)
    feats, tgts = [], []
    for seed, path in scene_files(seeds, width, height, nobj):
        t0 = time.time()
        fr = DeferredFrame(gpu, seed, width, height, nobj, path=path)
        os.remove(path)
        f, t = fr.features(gpu)
        idx = torch.nonzero(fr.covered).reshape(-1)
        pick = idx[torch.randperm(len(idx), generator=g, device="cuda")[:per_seed]]
        feats.append(f[pick].clone())
        tgts.append(t[pick].clone())
        del f, t, fr
        if log:
            log("seed %d: %d covered pixels, %d samples (%.1fs)" % (seed, len(idx), len(pick), time.time() - t0))
    return torch.cat(feats), torch.cat(tgts)


def train(gpu, net, features, targets, steps=20000, batch=8192, lr=2e-3, lr_final=2e-5, seed=0, log=None):
    """Adam with a cosine learning-rate decay; batches drawn uniformly with
    replacement.  Returns the per-step mean squared errors (every 100th)."""
    import math
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    n = features.shape[0]
    losses = []
    for s in range(steps):
        rate = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * s / max(1, steps - 1)))
        idx = torch.randint(0, n, (batch,), generator=g, device="cuda", dtype=torch.int32)
        net.train_step(gpu, features, targets, idx, rate)
        if s % 100 == 0 or s == steps - 1:
            losses.append(net.loss.item() / (3 * batch))
            if log and s % 2000 == 0:
                log("step %d lr %.2e mse %.3e" % (s, rate, losses[-1]))
    return losses


# ---- evaluation ----
def srgb_channels(c):
    """(H*W,) 0x00RRGGBB -> (H*W, 3) int."""
    c = np.asarray(c).astype(np.int64) & 0xffffff
    return np.stack([(c >> 16) & 255, (c >> 8) & 255, c & 255], -1)


def psnr(a, b):
    """PSNR in dB and max abs error of two packed sRGB8 images over all pixels."""
    d = srgb_channels(a) - srgb_channels(b)
    mse = float((d.astype(np.float64) ** 2).mean())
    return (float("inf") if mse == 0 else 10 * np.log10(255.0 ** 2 / mse)), int(np.abs(d).max())


def srgb8_table():
    """The library's sRGB8 encode table (26624 entries: the correctly rounded
    sRGB value of the midpoint of each exponent / top-11-mantissa-bit class
    of the clamped input), as the host runtime builds it."""
    k = np.arange(26624, dtype=np.uint32)
    x = ((((k + ((127 - 13) << 11)) << 12) | 0x800).astype(np.uint32)).view(np.float32).astype(np.float64)
    s = np.where(x <= 0.0031308, 12.92 * x, 1.055 * np.power(x, 1.0 / 2.4) - 0.055)
    return np.clip(np.floor(s * 255.0 + 0.5), 0, 255).astype(np.uint8)


def pack_srgb_torch(lin, lut):
    """Linear RGB -> 0x00RRGGBB through the library's sRGB8 table (torch)."""
    import torch
    lo = 2.0 ** -13
    c = lin.clamp(lo, float(np.frombuffer(np.uint32(0x3f7fffff).tobytes(), np.float32)[0]))
    idx = (c.contiguous().view(torch.int32) >> 12) - ((127 - 13) << 11)
    q = lut[idx.long()].to(torch.int64)
    return (q[:, 0] << 16) | (q[:, 1] << 8) | q[:, 2]


def evaluate(gpu, net, seeds, width=1920, height=1080, nobj=2_000_000, max_tile_mse=PSNR_40DB_MSE, log=None):
    """Per eval seed: PSNR / max-abs of the gated learned shader, of the
    trained network without fallback and of the untrained network (the
    virtual-light method alone), each against the plain shader (packed sRGB8
    over all pixels), and the share of covered tiles the network served."""
    import torch
    untrained = LearnedShader(seed=0)
    rows = []
    for seed, path in scene_files(seeds, width, height, nobj):
        fr = DeferredFrame(gpu, seed, width, height, nobj, path=path)
        os.remove(path)
        n = width * height
        plain = torch.zeros(n, dtype=torch.int32, device="cuda")
        fr.shade_plain(gpu, plain)
        status = torch.zeros(fr.ntiles, dtype=torch.uint8, device="cuda")
        res = {"seed": seed}
        for name, nt, thr in (("learned", net, max_tile_mse), ("network_only", net, float("inf")),
                              ("virtual_light", untrained, float("inf"))):
            o = torch.zeros(n, dtype=torch.int32, device="cuda")
            fr.shade_learned(gpu, nt, thr, o, tile_status=status if name == "learned" else None)
            gpu.shade_learned_check()
            res[name] = psnr(o.cpu().numpy(), plain.cpu().numpy())
            if name == "learned":
                st = status.cpu().numpy()
                res["served_tiles"] = float((st == 0).sum() / max(1, (st != 2).sum()))
        rows.append(res)
        if log:
            log(json.dumps(res))
    return rows


def main(argv=None):
    """python -m rsr_gb300.learned: trains the learned shader on the GPU and
    writes its weights (with the training and evaluation record)."""
    import argparse
    import torch
    from .gpu import GPU

    def seeds(s):
        a, _, b = s.partition("-")
        return list(range(int(a), int(b or a) + 1))

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--train-seeds", type=seeds, default=seeds("1-32"))
    ap.add_argument("--eval-seeds", type=seeds, default=seeds("100-107"))
    ap.add_argument("--samples", type=int, default=1 << 22)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--nobj", type=int, default=2_000_000)
    ap.add_argument("--out", default=WEIGHTS_PATH)
    a = ap.parse_args(argv)
    log = lambda s: print(s, flush=True)
    gpu = GPU(0)
    gpu.InstallDefaults()
    t0 = time.time()
    per_seed = a.samples // len(a.train_seeds)
    feats, tgts = collect_samples(gpu, a.train_seeds, per_seed, a.width, a.height, a.nobj, log=log)
    t1 = time.time()
    net = LearnedShader(seed=0)
    torch.cuda.synchronize()
    losses = train(gpu, net, feats, tgts, a.steps, a.batch, a.lr, log=log)
    torch.cuda.synchronize()
    t2 = time.time()
    log("data %.1fs, training %.1fs (%d steps of %d)" % (t1 - t0, t2 - t1, a.steps, a.batch))
    rows = evaluate(gpu, net, a.eval_seeds, a.width, a.height, a.nobj, log=log)
    meta = {"train_seeds": a.train_seeds, "samples": int(feats.shape[0]), "steps": a.steps, "batch": a.batch,
            "lr": a.lr, "size": [a.width, a.height], "nobj": a.nobj, "final_mse": losses[-1],
            "train_seconds": t2 - t1, "eval": rows}
    net.save(a.out, meta)
    log("saved %s" % a.out)
    gpu.close()


if __name__ == "__main__":
    main()
