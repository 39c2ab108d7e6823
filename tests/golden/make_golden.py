"""Generates tests/golden/frames.json, textures.json and postfx.json from
rsr's own CPU code.

Runs oracle/_ref/librsrref.so (rsr's sources built by oracle/ref/Makefile,
x86-64 only) on the seeded scenes of GOLDEN_SCENES and records, per scene
and gamma setting, SHA-256 digests of the sRGB8/linear colour buffer, the fp32
depth buffer, the canonical per-tile command streams, and the clipped vertex
buffer (coordinates + the program's varyings); the frames with float colour
stores (FLOAT_STORE_SCENES) record every output.  textures.json holds the
digests of textures built by rsr's image-loader path (TEXTURE_CASES: the
sRGB8 decode of PNGToTexture and Texture::maybe_make_mipmap), postfx.json
those of KawaseBlurFilter and Filter<GlowShader> on seeded canvases
(POSTFX_CASES).  The oracle is
checked against these digests on every machine, including ones without the
reference.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from rsr_gb300 import scenes  # noqa: E402

# name -> (factory, kwargs, varyings kept per clipped vertex)
GOLDEN_SCENES = {
    "plain_640_t64": ("plain_raster", {}, 3),
    "plain_320_t8": ("plain_raster", dict(seed=7, ntris=2000, width=320, height=180, tile_blocks=(1, 1)), 3),
    "plain_1080_t128": ("plain_raster", dict(seed=8, ntris=500, width=1920, height=1080, tile_blocks=(16, 16)), 3),
    "plain_640_t16x32": ("plain_raster", dict(seed=9, ntris=3000, width=640, height=360, tile_blocks=(2, 4)), 3),
    "sphere_1080_t32": ("textured_sphere", dict(divs=6), 2),
    # the benchmarked frame itself: seed 1, 7 subdivisions (327 680 triangles),
    # 1920x1080, 32 px tiles, 1024x1024 texture
    "sphere_1080_t32_d7": ("textured_sphere", dict(seed=1, divs=7, width=1920, height=1080, tile_blocks=(4, 4),
                                                   tex_dim=1024), 2),
    "clip_640_t64": ("clip_stress", {}, 3),
    "clip_2160_t32": ("clip_stress", dict(seed=5, width=3840, height=2160, tile_blocks=(4, 4), extent=3.0), 3),
    "mixed_640_t32": ("mixed_states", {}, 3),
    # scissor-enabled draws: odd rectangle edges, off screen, whole screen,
    # empty, depth writes off, clipped triangles; both attachment layouts
    "scissor_640_t32": ("scissor_scene", {}, 3),
    "scissor_640_t8_color_depth": ("scissor_scene", dict(seed=62, tile_blocks=(1, 1), color_depth=True), 3),
    "scissor_360_t64": ("scissor_scene", dict(seed=63, width=360, height=202, tile_blocks=(8, 8)), 3),
    # geometry of the deferred (G-buffer) scene drawn with the Gouraud program:
    # pins the G-buffer pass's depth to rsr
    "deferred_gouraud_640": ("deferred_scene", dict(nobj=20000, width=640, height=360, gouraud=True), 3),
    # instanced draws: ManyProgram cubes (per-instance matrices, some clipped)
    # and an instanced Gouraud DrawArraysInstanced
    "instanced_640_t32": ("instanced_scene", {}, 2),
    "instanced_320_t8_nocull": ("instanced_scene", dict(cull=False, seed=42, ninst=500, width=320, height=180,
                                                         tile_blocks=(1, 1)), 2),
    "instanced_720_t64": ("instanced_scene", dict(seed=43, ninst=3000, width=1280, height=720, tile_blocks=(8, 8)), 2),
    # OBJ1Program: per-vertex view-space lighting (sqrt, RSQRTPS, divide),
    # 1P and 2P binning, one sphere clipped at the near plane
    "obj1_640_t32": ("obj1_scene", {}, 3),
    "obj1_320_t8_2p": ("obj1_scene", dict(dense_hint=True, seed=52, width=320, height=180, tile_blocks=(1, 1)), 3),
    "obj1_720_t64": ("obj1_scene", dict(seed=53, nspheres=60, width=1280, height=720, tile_blocks=(8, 8)), 3),
}


# frames with rsr's float colour stores (StoreColor to FloatingPointCanvas,
# downsampled or not, and to QFloat4Canvas): name -> float_store_frame kwargs
FLOAT_STORE_SCENES = {
    "float_store_rgbf32": {},
    "float_store_rgbf32_mid": dict(mid=True),
    "float_store_color_depth": dict(color_depth=True),
    "float_store_color_depth_mid": dict(color_depth=True, mid=True),
}


def render_float_store(renderer, sc, gamma):
    """Renders a scenes.FloatStoreScene; returns {output: digest} plus the tile streams' digest."""
    for v in sc.outputs.values():
        v[:] = 0
    renderer.render_gl(sc.record(gamma=gamma), sc.width, sc.height, sc.tile_blocks)
    out = {k: digest(np.ascontiguousarray(v).view(np.uint32).tobytes()) for k, v in sc.outputs.items()}
    out["tiles"] = digest(b"".join(len(t).to_bytes(4, "little") + t for t in renderer.tiles()))
    return out


# textures built the way rsr's image loader builds them (PNGToTexture's
# conversion, Texture::maybe_make_mipmap): name -> (edge x, edge y, premultiply, seed)
TEXTURE_CASES = {
    "tex_1": (1, 1, 0, 1),
    "tex_2_premul": (2, 2, 1, 2),
    "tex_32": (32, 32, 0, 3),
    "tex_64_premul": (64, 64, 1, 4),
    "tex_512": (512, 512, 0, 5),
    "tex_128x64_nochain": (128, 64, 1, 6),
    "tex_48_nochain": (48, 48, 0, 7),
}


def texture_bytes(w, h, seed):
    """Seeded RGBA8 pixels (splitmix64 uniforms scaled to bytes)."""
    u = scenes.uniform01(seed * 7 + 1000, w * h * 4)
    return np.minimum((u * np.float32(256.0)).astype(np.int32), 255).astype(np.uint8)


def texture_digest(texels, power):
    return {"texels": digest(np.ascontiguousarray(texels).view(np.uint32).tobytes()), "power": int(power),
            "count": int(texels.shape[0])}


# post-processing of seeded float canvases by rsr's KawaseBlurFilter and
# Filter<GlowShader>: name -> (kind, width, height, distance or sRGB flag, seed)
POSTFX_CASES = {
    "kawase_2x2_d0": ("kawase", 2, 2, 0, 1),
    "kawase_61x37_d1": ("kawase", 61, 37, 1, 2),
    "kawase_160x90_d3": ("kawase", 160, 90, 3, 3),
    "kawase_96x54_d30": ("kawase", 96, 54, 30, 4),
    "glow_64x36_linear": ("glow", 64, 36, 0, 5),
    "glow_320x180_srgb": ("glow", 320, 180, 1, 6),
}


def postfx_inputs(kind, w, h, seed):
    """Seeded canvases: kawase an RGBA float (h, w, 4) source in [-1, 3);
    glow a quads canvas (h/2, w/2, 16) in [0, 1.5) and a blur (h/2, w/2, 4) in [0, 1.2)."""
    if kind == "kawase":
        return (scenes.uniform01(seed * 11 + 2000, h * w * 4).reshape(h, w, 4) * np.float32(4.0) - np.float32(1.0),)
    q = scenes.uniform01(seed * 11 + 3000, (h // 2) * (w // 2) * 16).reshape(h // 2, w // 2, 16) * np.float32(1.5)
    b = scenes.uniform01(seed * 11 + 4000, (h // 2) * (w // 2) * 4).reshape(h // 2, w // 2, 4) * np.float32(1.2)
    return q, b


def run_postfx(renderer, name):
    kind, w, h, arg, seed = POSTFX_CASES[name]
    ins = postfx_inputs(kind, w, h, seed)
    if kind == "kawase":
        return renderer.kawase(ins[0], arg)
    return renderer.glow(ins[0], ins[1], w, h, arg)


def make_scene(name):
    fn, kw, _ = GOLDEN_SCENES[name]
    kw = dict(kw)
    if "tile_blocks" in kw:
        kw["tile_blocks"] = tuple(kw["tile_blocks"])
    return getattr(scenes, fn)(**kw)


def digest(b):
    return hashlib.sha256(b).hexdigest()


def frame_digests(color, depth, tiles, clipped, nvary):
    return {
        "color": digest(np.ascontiguousarray(color).tobytes()),
        "depth": digest(np.ascontiguousarray(depth).view(np.uint32).tobytes()),
        "tiles": digest(b"".join(len(t).to_bytes(4, "little") + t for t in tiles)),
        "clipped": digest(np.ascontiguousarray(clipped[:, :4 + nvary]).view(np.uint32).tobytes()),
        "nclipped": int(clipped.shape[0]),
        "covered": int((depth < 1.0).sum()),
    }


def main():
    import oracle
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref/librsrref.so is not built (x86-64 host with the reference needed)")
    ref = oracle.CpuRenderer("ref")
    out = {}
    for name, (_, _, nvary) in GOLDEN_SCENES.items():
        sc = make_scene(name)
        for gamma in (False, True):
            c, d = ref.render(sc, gamma)
            out["%s/gamma%d" % (name, int(gamma))] = frame_digests(c, d, ref.tiles(), ref.clipped(), nvary)
            print(name, gamma, out["%s/gamma%d" % (name, int(gamma))]["covered"])
    for name, kw in FLOAT_STORE_SCENES.items():
        sc = scenes.float_store_frame(**kw)
        for gamma in (False, True):
            out["%s/gamma%d" % (name, int(gamma))] = render_float_store(ref, sc, gamma)
            print(name, gamma)
    with open(os.path.join(HERE, "frames.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    tex = {}
    for name, (w, h, pm, seed) in TEXTURE_CASES.items():
        texels, power = ref.texture_from_rgba8(texture_bytes(w, h, seed), w, h, pm)
        tex[name] = texture_digest(texels, power)
        print(name, power)
    with open(os.path.join(HERE, "textures.json"), "w") as f:
        json.dump(tex, f, indent=1, sort_keys=True)
    post = {name: digest(np.ascontiguousarray(run_postfx(ref, name)).view(np.uint32).tobytes())
            for name in POSTFX_CASES}
    with open(os.path.join(HERE, "postfx.json"), "w") as f:
        json.dump(post, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
