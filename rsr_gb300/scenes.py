"""Seeded synthetic scenes for the rasteriser path.

RNG: splitmix64(seed); each draw u = (x >> 40) * 2^-24 in float32 and a value
in [a, b) is a + (b - a) * u, also in float32.  Values are generated per
triangle, per vertex, then per field in the listed order.  The same bytes
feed the reference, the oracle and the GPU library.

Scenes:
  plain_raster      640x360, 10 000 random NDC triangles, Gouraud, no culling
  textured_sphere   1920x1080, icosphere (subdivision 7: 327 680 triangles),
                    60 degree camera at distance 3, back-face culling,
                    1024x1024 value-noise texture with bilinear sampling
Every scene ends with a STORE_COLOR (sRGB8) and STORE_DEPTH (fp32).
"""
import math

import numpy as np

from . import abi
from .gl import GL

GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(seed, n):
    """The first n outputs of splitmix64(seed) as uint64."""
    with np.errstate(over="ignore"):
        i = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed) + i * GOLDEN
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed, n):
    return ((splitmix64(seed, n) >> np.uint64(40)).astype(np.float32)
            * np.float32(1.0 / (1 << 24)))


def lerp(a, b, u):
    return (np.float32(a) + (np.float32(b) - np.float32(a)) * u).astype(np.float32)


def pad4(a, fill=0.0):
    n = (len(a) + 3) & ~3
    out = np.full(n, fill, np.float32)
    out[:len(a)] = a
    return out


# ---- matrices (column-major, rmlm::mat4::ff) ----
def mat_from_rows(rows):
    """rmlm::mat4's 16-float constructor takes rows (rmlm_mat4.hxx); ff is column-major."""
    return np.asarray(rows, np.float32).reshape(4, 4).T.reshape(16).copy()


def look_at(eye, center, up):
    eye, center, up = (np.asarray(v, np.float64) for v in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    rot = np.array([[s[0], s[1], s[2], 0], [u[0], u[1], u[2], 0],
                    [-f[0], -f[1], -f[2], 0], [0, 0, 0, 1]])
    tr = np.eye(4)
    tr[:3, 3] = -eye
    return mat_from_rows(rot @ tr)


def perspective(fovy_deg, aspect, znear, zfar):
    h = math.tan(math.radians(fovy_deg) / 2) * znear
    w = h * aspect
    l, r, b, t, n, f = -w, w, -h, h, znear, zfar
    rows = [[2 * n / (r - l), 0, (r + l) / (r - l), 0],
            [0, 2 * n / (t - b), (t + b) / (t - b), 0],
            [0, 0, -(f + n) / (f - n), -2 * f * n / (f - n)],
            [0, 0, -1, 0]]
    return mat_from_rows(rows)


class Scene:
    """A frame description: dimensions, tile size, and a recorder callback.

    `arrays` holds the host inputs by name; `record(gl, ref)` writes the frame
    into a GL using ref(name) to obtain the buffer object to point at (the
    numpy array itself, or a device tensor holding a copy of it)."""

    def __init__(self, name, width, height, tile_blocks, arrays, record_fn, ntris, post_program=None,
                 store_depth=True):
        self.post_program = post_program
        self.store_depth = store_depth   # RB_COLOR_DEPTH frames have no separate depth to store
        self.name = name
        self.width = width
        self.height = height
        self.tile_blocks = tile_blocks
        self.arrays = arrays
        self._record = record_fn
        self.ntris = ntris
        self.color = np.zeros(width * height, np.uint32)
        self.depth = np.zeros(width * height, np.float32)

    def record(self, ref=None, color=None, depth=None, gamma=True):
        gl = GL()
        ref = ref or (lambda k: self.arrays[k])
        self._record(gl, ref)
        if self.post_program is None:
            gl.UseProgram(abi.PROGRAM_DEFAULT_POST)
        gl.StoreColor(self.color if color is None else color, self.width, self.height, gamma)
        if self.store_depth:
            gl.StoreDepth(self.depth if depth is None else depth)
        return gl


def _begin_frame(gl, clear_rgb=(0.0, 0.0, 0.0)):
    gl.RenderbufferType(abi.GL_COLOR_ATTACHMENT0, abi.RB_RGBF32)
    gl.RenderbufferType(abi.GL_DEPTH_ATTACHMENT, abi.RB_F32)
    gl.ClearColor(clear_rgb)
    gl.ClearDepth(1.0)
    gl.Clear(abi.GL_COLOR_BUFFER_BIT | abi.GL_DEPTH_BUFFER_BIT)


def plain_raster(seed=0, ntris=10000, width=640, height=360, tile_blocks=(8, 8), spread=1.0, clear_rgb=(0.0, 0.0, 0.0)):
    """Random NDC triangles (xyz in [-1,1], w=1), rgb in [0,1], Gouraud, LESS,
    no culling; DrawElements of sequential indices.  spread < 1 shrinks each
    triangle about its own centre: centre uniform in [-(1-s), 1-s]^3 and
    vertices at centre + s * U[-1,1]^3, so positions stay in [-1,1] and the
    expected screen area scales by s^2 (spread 1 is the unscaled generator)."""
    nverts = 3 * ntris
    u = uniform01(seed, nverts * 6).reshape(ntris, 3, 6)
    pos = lerp(-1.0, 1.0, u[:, :, 0:3])
    if spread < 1.0:
        c = lerp(-(1.0 - spread), 1.0 - spread, uniform01(seed + 0x5EED, ntris * 3).reshape(ntris, 1, 3))
        pos = c + spread * pos
    pos = pos.reshape(nverts, 3)
    rgb = lerp(0.0, 1.0, u[:, :, 3:6]).reshape(nverts, 3)
    # a draw holds at most 32766 vertices (u16 indices, bit 15 = back-face flag):
    # larger sets are drawn as consecutive draws of 10922 triangles
    per_draw = min(ntris, 10922)
    arrays = {
        "px": pad4(pos[:, 0]), "py": pad4(pos[:, 1]), "pz": pad4(pos[:, 2]),
        "cr": pad4(rgb[:, 0]), "cg": pad4(rgb[:, 1]), "cb": pad4(rgb[:, 2]),
        "idx": np.arange(3 * per_draw, dtype=np.uint16),
    }

    def record(gl, ref):
        _begin_frame(gl, clear_rgb)
        gl.UseProgram(abi.PROGRAM_GOURAUD)
        if ntris <= per_draw:
            gl.UseBuffer(0, (ref("px"), ref("py"), ref("pz")))
            gl.UseBuffer(3, (ref("cr"), ref("cg"), ref("cb")))
            gl.DrawElements(nverts, ref("idx"), 0)
            return
        for first in range(0, ntris, per_draw):
            v0 = 3 * first
            gl.UseBuffer(0, tuple(ref(k)[v0:] for k in ("px", "py", "pz")))
            gl.UseBuffer(3, tuple(ref(k)[v0:] for k in ("cr", "cg", "cb")))
            gl.DrawElements(3 * min(per_draw, ntris - first), ref("idx"), 0)

    return Scene("plain_raster", width, height, tile_blocks, arrays, record, ntris)


BATCH_RESOLUTIONS = ((320, 180), (640, 360), (1280, 720), (1920, 1080), (3840, 2160))


def batch_frames(seed=0, nframes=64, tris=(1_000, 1_000_000), resolutions=BATCH_RESOLUTIONS):
    """Config-4 batch: nframes plain_raster frames (the config-1 generator,
    frame i seeded seed * 1000 + i), triangle counts log-uniform in
    [tris[0], tris[1]], resolutions drawn uniformly from `resolutions`.
    Frames above 10 000 triangles shrink their triangles by sqrt(10 000 / n)
    (plain_raster spread), which keeps the expected overdraw at that of the
    10 000-triangle config-1 frame: unscaled, one 1M-triangle 3840x2160 frame
    needs about 2e9 tile-list entries and 6e11 pixel tests."""
    u = uniform01(seed + 7_000_001, nframes * 2).reshape(nframes, 2)
    lo, hi = np.log(tris[0]), np.log(tris[1])
    counts = np.rint(np.exp(lerp(lo, hi, u[:, 0]))).astype(np.int64)
    pick = np.minimum((u[:, 1] * len(resolutions)).astype(np.int64), len(resolutions) - 1)
    out = []
    for i in range(nframes):
        w, h = resolutions[int(pick[i])]
        n = int(counts[i])
        out.append(plain_raster(seed=seed * 1000 + i, ntris=n, width=w, height=h, tile_blocks=(4, 4),
                                spread=min(1.0, float(np.sqrt(10_000.0 / n)))))
    return out


# ---- icosphere ----
def icosphere(divs):
    """Unit icosphere: vertices (float32, normalised) and CCW-outward triangles."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
             (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
             (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
             (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(divs):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]
        nf = []
        for (a, b, c) in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (ab, b, bc), (ab, bc, ca), (ca, bc, c)]
        faces = nf
    return np.array(verts, np.float32), np.array(faces, np.int64)


def value_noise_rgba8(seed, dim=1024, cells=(8, 16, 32, 64)):
    """Seeded multi-octave value noise, RGBA8 (alpha = 255)."""
    img = np.zeros((dim, dim, 3), np.float64)
    total = 0.0
    for k, c in enumerate(cells):
        lat = uniform01(seed * 7919 + k + 1, (c + 1) * (c + 1) * 3).reshape(c + 1, c + 1, 3).astype(np.float64)
        lat[c, :, :] = lat[0, :, :]
        lat[:, c, :] = lat[:, 0, :]
        g = (np.arange(dim) + 0.5) * c / dim
        i0 = np.floor(g).astype(int)
        f = g - i0
        f = f * f * (3 - 2 * f)
        a = lat[i0][:, i0] * (1 - f)[None, :, None] + lat[i0][:, i0 + 1] * f[None, :, None]
        b = lat[i0 + 1][:, i0] * (1 - f)[None, :, None] + lat[i0 + 1][:, i0 + 1] * f[None, :, None]
        layer = a * (1 - f)[:, None, None] + b * f[:, None, None]
        w = 1.0 / (1 << k)
        img += w * layer
        total += w
    rgb = np.clip(np.round(img / total * 255.0), 0, 255).astype(np.uint8)
    out = np.full((dim, dim, 4), 255, np.uint8)
    out[:, :, :3] = rgb
    return out


def srgb8_to_linear(c):
    c = c.astype(np.float64) / 255.0
    return np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4).astype(np.float32)


def make_mip_chain(rgba):
    """Stacked mip chain as rglr::Texture::maybe_make_mipmap builds it
    (rglr_texture.cxx:33-80): level 0 in rows [0, W), each next level below
    the previous one with the same row stride; each texel the float32 sum of
    its 2x2 parents ((a+b)+c)+d divided by 4."""
    dim = rgba.shape[0]
    buf = np.zeros((2 * dim, dim, 4), np.float32)
    buf[:dim] = rgba
    src_row, size = 0, dim
    dst_row = dim
    while size > 1:
        s = buf[src_row:src_row + size, :size]
        a, b = s[0::2, 0::2], s[0::2, 1::2]
        c, d = s[1::2, 0::2], s[1::2, 1::2]
        buf[dst_row:dst_row + size // 2, :size // 2] = (((a + b) + c) + d) / np.float32(4.0)
        src_row = dst_row
        dst_row += size // 2
        size //= 2
    return buf.reshape(-1)


def textured_sphere(seed=1, divs=7, width=1920, height=1080, tile_blocks=(4, 4), tex_dim=1024):
    """AmyProgram on an icosphere, chunked into draws of at most 32767 vertices."""
    verts, faces = icosphere(divs)
    # spherical uv
    uu = (np.arctan2(verts[:, 2], verts[:, 0]) / (2 * np.pi) + 0.5).astype(np.float32)
    vv = (np.arcsin(np.clip(verts[:, 1], -1, 1)) / np.pi + 0.5).astype(np.float32)
    arrays = {}
    draws = []
    start = 0
    nfaces = len(faces)
    while start < nfaces:
        local = {}
        end = start
        while end < nfaces:
            new = [v for v in faces[end] if v not in local]
            if len(local) + len(new) > 32764:
                break
            for v in new:
                local[v] = len(local)
            end += 1
        gidx = np.fromiter(local.keys(), np.int64, len(local))
        k = len(draws)
        arrays["px%d" % k] = pad4(verts[gidx, 0])
        arrays["py%d" % k] = pad4(verts[gidx, 1])
        arrays["pz%d" % k] = pad4(verts[gidx, 2])
        arrays["u%d" % k] = pad4(uu[gidx])
        arrays["v%d" % k] = pad4(vv[gidx])
        arrays["idx%d" % k] = np.array([local[v] for f in faces[start:end] for v in f], np.uint16)
        draws.append((k, 3 * (end - start)))
        start = end
    rgba8 = value_noise_rgba8(seed, tex_dim)
    lin = np.empty((tex_dim, tex_dim, 4), np.float32)
    lin[:, :, :3] = srgb8_to_linear(rgba8[:, :, :3])
    lin[:, :, 3] = rgba8[:, :, 3].astype(np.float32) / np.float32(255.0)
    arrays["tex"] = make_mip_chain(lin)
    view = look_at((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0))
    proj = perspective(60.0, width / height, 0.1, 100.0)

    def record(gl, ref):
        _begin_frame(gl, (0.1, 0.1, 0.1))
        gl.UseProgram(abi.PROGRAM_AMY)
        gl.Enable(abi.GL_CULL_FACE)
        gl.CullFace(abi.GL_BACK)
        gl.ViewMatrix(view)
        gl.ProjectionMatrix(proj)
        gl.BindTexture(0, ref("tex"), tex_dim, tex_dim, tex_dim, abi.GL_LINEAR_MIPMAP_NEAREST)
        for k, count in draws:
            gl.UseBuffer(0, (ref("px%d" % k), ref("py%d" % k), ref("pz%d" % k)))
            gl.UseBuffer(9, ref("u%d" % k))
            gl.UseBuffer(10, ref("v%d" % k))
            gl.DrawElements(count, ref("idx%d" % k), abi.RGL_HINT_DENSE | abi.RGL_HINT_READ4)

    return Scene("textured_sphere", width, height, tile_blocks, arrays, record, nfaces)


def clip_stress(seed=3, ntris=3000, width=640, height=360, tile_blocks=(8, 8), extent=6.0):
    """Random triangles around a perspective camera at the origin: many cross
    the near plane or the guard band and go through the Sutherland-Hodgman
    clipper and the scalar rasteriser.  Culling of back faces is on so the
    clipper's winding handling is exercised too."""
    nverts = 3 * ntris
    u = uniform01(seed, nverts * 6).reshape(ntris, 3, 6)
    pos = lerp(-extent, extent, u[:, :, 0:3]).reshape(nverts, 3)
    rgb = lerp(0.0, 1.0, u[:, :, 3:6]).reshape(nverts, 3)
    arrays = {
        "px": pad4(pos[:, 0]), "py": pad4(pos[:, 1]), "pz": pad4(pos[:, 2]),
        "cr": pad4(rgb[:, 0]), "cg": pad4(rgb[:, 1]), "cb": pad4(rgb[:, 2]),
        "idx": np.arange(nverts, dtype=np.uint16),
    }
    proj = perspective(90.0, width / height, 0.5, 50.0)

    def record(gl, ref):
        _begin_frame(gl)
        gl.UseProgram(abi.PROGRAM_GOURAUD)
        gl.Enable(abi.GL_CULL_FACE)
        gl.CullFace(abi.GL_BACK)
        gl.ProjectionMatrix(proj)
        gl.UseBuffer(0, (ref("px"), ref("py"), ref("pz")))
        gl.UseBuffer(3, (ref("cr"), ref("cg"), ref("cb")))
        gl.DrawElements(nverts, ref("idx"), 0)

    return Scene("clip_stress", width, height, tile_blocks, arrays, record, ntris)


def mixed_states(seed=13, width=640, height=360, tile_blocks=(4, 4)):
    """Several draws with different states in one frame: opaque Gouraud with
    LESS, a textured sphere with alpha blending (texture alpha from noise),
    Gouraud with LEQUAL, Gouraud with depth writes off, then an exposure
    post program for the store.  Exercises every ordering rule of the tile
    interpreter and the switches between them."""
    n1, n2, n3 = 1500, 800, 600
    u = uniform01(seed, (n1 + n2 + n3) * 3 * 6).reshape(-1, 3, 6)
    arrays = {}

    def tri_set(tag, rows, zlo, zhi):
        pos = np.concatenate([lerp(-1.0, 1.0, rows[:, :, 0:2]), lerp(zlo, zhi, rows[:, :, 2:3])], -1).reshape(-1, 3)
        rgb = lerp(0.0, 1.0, rows[:, :, 3:6]).reshape(-1, 3)
        for k, c in enumerate("xyz"):
            arrays["%s_p%s" % (tag, c)] = pad4(pos[:, k])
        for k, c in enumerate("rgb"):
            arrays["%s_c%s" % (tag, c)] = pad4(rgb[:, k])
        arrays["%s_idx" % tag] = np.arange(len(pos), dtype=np.uint16)
        return len(pos)

    c1 = tri_set("a", u[:n1], -1.0, 1.0)
    c3 = tri_set("c", u[n1:n1 + n2], -0.5, 0.5)
    c4 = tri_set("d", u[n1 + n2:], -1.0, 0.0)
    verts, faces = icosphere(3)
    uu = (np.arctan2(verts[:, 2], verts[:, 0]) / (2 * np.pi) + 0.5).astype(np.float32)
    vv = (np.arcsin(np.clip(verts[:, 1], -1, 1)) / np.pi + 0.5).astype(np.float32)
    arrays["s_px"], arrays["s_py"], arrays["s_pz"] = (pad4(verts[:, k]) for k in range(3))
    arrays["s_u"], arrays["s_v"] = pad4(uu), pad4(vv)
    arrays["s_idx"] = faces.reshape(-1).astype(np.uint16)
    rgba8 = value_noise_rgba8(seed, 64, cells=(4, 8))
    alpha = value_noise_rgba8(seed + 1, 64, cells=(4,))[:, :, 0]
    lin = np.empty((64, 64, 4), np.float32)
    lin[:, :, :3] = srgb8_to_linear(rgba8[:, :, :3])
    lin[:, :, 3] = alpha.astype(np.float32) / np.float32(255.0)
    arrays["tex"] = make_mip_chain(lin)
    view = look_at((0.0, 0.0, 2.2), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0))
    proj = perspective(60.0, width / height, 0.1, 100.0)
    ident = np.eye(4, dtype=np.float32).reshape(16)

    def gouraud(gl, ref, tag, count):
        gl.UseProgram(abi.PROGRAM_GOURAUD)
        gl.UseBuffer(0, (ref(tag + "_px"), ref(tag + "_py"), ref(tag + "_pz")))
        gl.UseBuffer(3, (ref(tag + "_cr"), ref(tag + "_cg"), ref(tag + "_cb")))
        gl.DrawElements(count, ref(tag + "_idx"), 0)

    def record(gl, ref):
        _begin_frame(gl, (0.2, 0.1, 0.05))
        gouraud(gl, ref, "a", c1)                          # 0x6e2
        gl.UseProgram(abi.PROGRAM_AMY)                     # 0x6f2: alpha blending
        gl.Enable(abi.GL_BLEND)
        gl.Enable(abi.GL_CULL_FACE)
        gl.ViewMatrix(view)
        gl.ProjectionMatrix(proj)
        gl.BindTexture(0, ref("tex"), 64, 64, 64, abi.GL_LINEAR_MIPMAP_NEAREST)
        gl.UseBuffer(0, (ref("s_px"), ref("s_py"), ref("s_pz")))
        gl.UseBuffer(9, ref("s_u"))
        gl.UseBuffer(10, ref("s_v"))
        gl.DrawElements(len(faces) * 3, ref("s_idx"), abi.RGL_HINT_DENSE | abi.RGL_HINT_READ4)
        gl.Disable(abi.GL_BLEND)
        gl.Disable(abi.GL_CULL_FACE)
        gl.ViewMatrix(ident)
        gl.ProjectionMatrix(ident)
        gl.DepthFunc(abi.GL_LEQUAL)                        # 0x6e6
        gouraud(gl, ref, "c", c3)
        gl.DepthFunc(abi.GL_LESS)
        gl.DepthWriteMask(False)                           # 0x6c2
        gouraud(gl, ref, "d", c4)
        gl.DepthWriteMask(True)
        gl.UseProgram(abi.PROGRAM_EXPOSURE_POST)
        gl.UseUniforms([1.5])

    return Scene("mixed_states", width, height, tile_blocks, arrays, record,
                 c1 // 3 + len(faces) + c3 // 3 + c4 // 3, post_program=abi.PROGRAM_EXPOSURE_POST)


def scissor_scene(seed=61, width=640, height=360, tile_blocks=(4, 4), color_depth=False, past_edges=False):
    """Draws under scissor rectangles (GL::Scissor, GPU::ScissorRect with
    rsr's bottom = height - y - 1, rglv_gpu.hxx:258-276): an unscissored draw,
    then rectangles with odd edges that cut quads, one partly off screen (with
    blending), the whole-screen rectangle (whose last row the reference
    leaves out), an empty one, one with depth writes off, and near-plane
    clipped triangles under a scissor (the clipper's covered-tile walk).
    color_depth: RB_COLOR_DEPTH attachments (LESS only, with and without
    blending).  past_edges: one more rectangle reaching past the right and
    bottom edges of the target, where rsr bins to tile indices outside its
    grid (this library and the oracle keep to the grid)."""
    sets = {"a": 1200, "b": 600, "c": 400, "d": 400, "f": 200, "g": 300}
    u = uniform01(seed, sum(sets.values()) * 3 * 6).reshape(-1, 3, 6)
    arrays = {}
    at = 0
    counts = {}
    for tag, n in sets.items():
        rows = u[at:at + n]
        at += n
        pos = lerp(-1.0, 1.0, rows[:, :, 0:3]).reshape(-1, 3)
        rgb = lerp(0.0, 1.0, rows[:, :, 3:6]).reshape(-1, 3)
        for k, c in enumerate("xyz"):
            arrays["%s_p%s" % (tag, c)] = pad4(pos[:, k])
        for k, c in enumerate("rgb"):
            arrays["%s_c%s" % (tag, c)] = pad4(rgb[:, k])
        arrays["%s_idx" % tag] = np.arange(len(pos), dtype=np.uint16)
        counts[tag] = len(pos)
    # triangles around a perspective camera: many cross the near plane
    ne = 800
    ue = uniform01(seed + 1, ne * 3 * 6).reshape(ne, 3, 6)
    pos = lerp(-6.0, 6.0, ue[:, :, 0:3]).reshape(-1, 3)
    rgb = lerp(0.0, 1.0, ue[:, :, 3:6]).reshape(-1, 3)
    for k, c in enumerate("xyz"):
        arrays["e_p%s" % c] = pad4(pos[:, k])
    for k, c in enumerate("rgb"):
        arrays["e_c%s" % c] = pad4(rgb[:, k])
    arrays["e_idx"] = np.arange(len(pos), dtype=np.uint16)
    counts["e"] = len(pos)
    proj = perspective(90.0, width / height, 0.5, 50.0)
    ident = np.eye(4, dtype=np.float32).reshape(16)

    def draw(gl, ref, tag):
        gl.UseBuffer(0, (ref(tag + "_px"), ref(tag + "_py"), ref(tag + "_pz")))
        gl.UseBuffer(3, (ref(tag + "_cr"), ref(tag + "_cg"), ref(tag + "_cb")))
        gl.DrawElements(counts[tag], ref(tag + "_idx"), 0)

    def record(gl, ref):
        rb = abi.RB_COLOR_DEPTH if color_depth else abi.RB_RGBF32
        gl.RenderbufferType(abi.GL_COLOR_ATTACHMENT0, rb)
        gl.RenderbufferType(abi.GL_DEPTH_ATTACHMENT, abi.RB_COLOR_DEPTH if color_depth else abi.RB_F32)
        gl.ClearColor((0.05, 0.1, 0.2))
        gl.ClearDepth(1.0)
        gl.Clear(abi.GL_COLOR_BUFFER_BIT | abi.GL_DEPTH_BUFFER_BIT)
        gl.UseProgram(abi.PROGRAM_GOURAUD)
        draw(gl, ref, "a")                                   # no scissor
        gl.Enable(abi.GL_SCISSOR_TEST)
        gl.Scissor(37, 21, 101, 77)                          # odd edges on every side
        draw(gl, ref, "b")
        gl.Scissor(0, 0, width, height)                      # the whole screen
        if not color_depth:
            gl.DepthFunc(abi.GL_LEQUAL)
        draw(gl, ref, "c")
        gl.DepthFunc(abi.GL_LESS)
        gl.Scissor(-13, height - 41, 160, 90)                # partly off screen (left, top), blending
        gl.Enable(abi.GL_BLEND)
        draw(gl, ref, "d")
        gl.Disable(abi.GL_BLEND)
        gl.Scissor(10, 10, 0, 0)                             # empty
        draw(gl, ref, "f")
        if not color_depth:
            gl.Scissor(width // 2 - 63, height // 2 - 41, 127, 83)
            gl.DepthWriteMask(False)
            draw(gl, ref, "g")
            gl.DepthWriteMask(True)
        if past_edges:
            gl.Scissor(width - 37, -11, 100, 60)             # past the right and bottom edges
            draw(gl, ref, "b")
        gl.Scissor(201, 150, 173, 95)                        # clipped triangles
        gl.ProjectionMatrix(proj)
        gl.Enable(abi.GL_CULL_FACE)
        gl.CullFace(abi.GL_BACK)
        draw(gl, ref, "e")
        gl.Disable(abi.GL_CULL_FACE)
        gl.ProjectionMatrix(ident)
        gl.Disable(abi.GL_SCISSOR_TEST)

    ntris = sum(counts.values()) // 3 - (0 if not color_depth else counts["g"] // 3) + (counts["b"] // 3 if past_edges else 0)
    return Scene("scissor_scene", width, height, tile_blocks, arrays, record, ntris, store_depth=not color_depth)


# ---- deferred scene: many small objects, G-buffer program, 64 point lights ----
def _random_rotations(u):
    """Uniform random rotation matrices from three uniforms per object (Shoemake)."""
    u1, u2, u3 = (u[:, k].astype(np.float64) for k in range(3))
    a, b = np.sqrt(1 - u1), np.sqrt(u1)
    qx, qy = a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2)
    qz, qw = b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)
    r = np.empty((len(u), 3, 3))
    r[:, 0, 0] = 1 - 2 * (qy * qy + qz * qz); r[:, 0, 1] = 2 * (qx * qy - qz * qw); r[:, 0, 2] = 2 * (qx * qz + qy * qw)
    r[:, 1, 0] = 2 * (qx * qy + qz * qw); r[:, 1, 1] = 1 - 2 * (qx * qx + qz * qz); r[:, 1, 2] = 2 * (qy * qz - qx * qw)
    r[:, 2, 0] = 2 * (qx * qz - qy * qw); r[:, 2, 1] = 2 * (qy * qz + qx * qw); r[:, 2, 2] = 1 - 2 * (qx * qx + qy * qy)
    return r


def _cube_mesh():
    """Unit cube, 24 vertices (flat face normals), 12 CCW-outward triangles."""
    faces = [((1, 0, 0), (0, 1, 0)), ((-1, 0, 0), (0, 0, 1)), ((0, 1, 0), (0, 0, 1)),
             ((0, -1, 0), (1, 0, 0)), ((0, 0, 1), (1, 0, 0)), ((0, 0, -1), (0, 1, 0))]
    pos, nrm, tri = [], [], []
    for n, t in faces:
        n, t = np.array(n, float), np.array(t, float)
        b = np.cross(n, t)
        base = len(pos)
        for (su, sv) in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
            pos.append(0.5 * (n + su * t + sv * b))
            nrm.append(n)
        tri += [(base, base + 1, base + 2), (base, base + 2, base + 3)]
    return np.array(pos), np.array(nrm), np.array(tri)


def _morton3(p):
    q = np.clip(((p + 10.0) / 20.0 * 1023).astype(np.int64), 0, 1023)
    code = np.zeros(len(p), np.int64)
    for bit in range(10):
        for k in range(3):
            code |= ((q[:, k] >> bit) & 1) << (3 * bit + k)
    return code


def deferred_scene(nobj=2_000_000, seed=3, width=1920, height=1080, tile_blocks=(4, 4),
                   size=(0.05, 0.15), sphere_every=8, nlights=64, gouraud=False, arrays=None):
    """Config-3 G-buffer scene: nobj objects in [-10,10]^3 with random
    orientation and size (every sphere_every-th one an icosahedron with
    smooth normals, the others cubes with flat normals), random RGB albedo,
    drawn with the G-buffer program (chunked into <= 32760-vertex draws,
    objects in 3D Morton order of their centre), camera at (0,0,30) looking
    at the origin with a 60 degree field of view; plus nlights point lights
    (position in the box, colour in [0,1], radius in [2,6]).  gouraud=True
    draws the same geometry with the Gouraud test program (normals as colour)
    and ordinary colour/depth stores, so rsr itself can render it.
    arrays: the vertex arrays of an earlier call with the same seed and
    sizes (scene.arrays), which skips rebuilding them."""
    if arrays is not None:
        return _deferred_scene_record(arrays, None, None, None, nobj, seed, width, height, tile_blocks,
                                      sphere_every, nlights, gouraud)
    u = uniform01(seed, nobj * 10).reshape(nobj, 10)
    centre = lerp(-10.0, 10.0, u[:, 0:3]).astype(np.float64)
    rot = _random_rotations(u[:, 3:6])
    scale = lerp(size[0], size[1], u[:, 6]).astype(np.float64)
    rgb = np.clip((lerp(0.2, 1.0, u[:, 7:10]) * 255.0).astype(np.int64), 0, 255)
    order = np.argsort(_morton3(centre), kind="stable")
    centre, rot, scale, rgb = centre[order], rot[order], scale[order], rgb[order]
    return _deferred_scene_record(None, centre, rot, (scale, rgb), nobj, seed, width, height, tile_blocks,
                                  sphere_every, nlights, gouraud)


def _deferred_scene_record(arrays, centre, rot, scale_rgb, nobj, seed, width, height, tile_blocks,
                           sphere_every, nlights, gouraud):
    is_sphere = (np.arange(nobj) % sphere_every) == sphere_every - 1
    cpos, cnrm, ctri = _cube_mesh()
    iverts, ifaces = icosphere(0)
    ipos, inrm = iverts.astype(np.float64) * 0.6, iverts.astype(np.float64)
    build = arrays is None
    if build:
        arrays = {}
        scale, rgb = scale_rgb
    draws = []
    for kind, mpos, mnrm, mtri, sel in (("c", cpos, cnrm, ctri, ~is_sphere), ("s", ipos, inrm, ifaces, is_sphere)):
        n = int(sel.sum())
        if n == 0:
            continue
        nv = len(mpos)
        per_draw = 32760 // nv
        for first in range(0, n, per_draw):
            cnt = min(per_draw, n - first)
            draws.append((kind, first * nv, cnt * len(mtri) * 3))
        if not build:
            continue
        wp = np.einsum("oij,vj->ovi", rot[sel], mpos) * scale[sel][:, None, None] + centre[sel][:, None, :]
        wn = np.einsum("oij,vj->ovi", rot[sel], mnrm)
        alb = (rgb[sel][:, 0] | (rgb[sel][:, 1] << 8) | (rgb[sel][:, 2] << 16)).astype(np.float32)
        for k, c in enumerate("xyz"):
            arrays["%s_p%s" % (kind, c)] = pad4(wp[:, :, k].reshape(-1).astype(np.float32))
            arrays["%s_n%s" % (kind, c)] = pad4(wn[:, :, k].reshape(-1).astype(np.float32))
        arrays["%s_alb" % kind] = pad4(np.repeat(alb, nv))
        arrays["%s_idx" % kind] = (np.arange(per_draw)[:, None, None] * nv + mtri[None]).reshape(-1).astype(np.uint16)
    lu = uniform01(seed + 101, nlights * 7).reshape(nlights, 7)
    lights = np.zeros((nlights, 8), np.float32)
    lights[:, 0:3] = lerp(-10.0, 10.0, lu[:, 0:3])
    lights[:, 3] = lerp(2.0, 6.0, lu[:, 3])
    lights[:, 4:7] = lerp(0.0, 1.0, lu[:, 4:7])
    view = look_at((0.0, 0.0, 30.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0))
    proj = perspective(60.0, width / height, 1.0, 100.0)
    vp = proj.reshape(4, 4).T.astype(np.float64) @ view.reshape(4, 4).T.astype(np.float64)
    ivp = np.linalg.inv(vp).T.reshape(16).astype(np.float32)   # column-major inverse
    ntris = sum(c // 3 for _, _, c in draws)

    def record(gl, ref):
        gl.RenderbufferType(abi.GL_COLOR_ATTACHMENT0, abi.RB_RGBF32)
        gl.RenderbufferType(abi.GL_DEPTH_ATTACHMENT, abi.RB_F32)
        gl.ClearColor((0.0, 0.0, 0.0))
        gl.ClearDepth(1.0)
        gl.Clear(abi.GL_COLOR_BUFFER_BIT | abi.GL_DEPTH_BUFFER_BIT)
        gl.UseProgram(abi.PROGRAM_GOURAUD if gouraud else abi.PROGRAM_GBUFFER)
        gl.ViewMatrix(view)
        gl.ProjectionMatrix(proj)
        for kind, vbase, count in draws:
            gl.UseBuffer(0, tuple(ref("%s_p%s" % (kind, c), vbase) for c in "xyz"))
            gl.UseBuffer(3, tuple(ref("%s_n%s" % (kind, c), vbase) for c in "xyz"))
            if not gouraud:
                gl.UseBuffer(6, ref("%s_alb" % kind, vbase))
            gl.DrawElements(count, ref("%s_idx" % kind, 0), 0)

    if gouraud:
        sc = Scene("deferred_gouraud", width, height, tile_blocks, arrays,
                   lambda gl, ref: record(gl, lambda k, off=0: ref(k)[off:]), ntris)
        return sc
    sc = DeferredScene("deferred", width, height, tile_blocks, arrays, record, ntris)
    sc.lights, sc.ivp, sc.eye, sc.nobj, sc.ndraws = lights, ivp, np.array([0.0, 0.0, 30.0], np.float32), nobj, len(draws)
    return sc


class DeferredScene(Scene):
    """A G-buffer frame.  record(ref, gbuffer=...) takes ref(name, offset)
    (element offset into the named array) and the five G-buffer planes."""

    def __init__(self, *a, **kw):
        super().__init__(*a, **kw)
        n = self.width * self.height
        self.gbuf = {"depth": np.zeros(n, np.float32), "nx": np.zeros(n, np.uint16), "ny": np.zeros(n, np.uint16),
                     "nz": np.zeros(n, np.uint16), "albedo": np.zeros(n, np.uint32)}

    def record(self, ref=None, gbuffer=None, **_):
        gl = GL()
        if ref is None:
            def ref(k, off=0):
                return self.arrays[k][off:]
        g = gbuffer or self.gbuf
        self._record(gl, ref)
        gl.StoreGBuffer(g["depth"], g["nx"], g["ny"], g["nz"], g["albedo"], self.width, self.height)
        return gl


class FloatStoreScene(Scene):
    """A frame whose colour also leaves through rsr's float stores:
    StoreColor(FloatingPointCanvas*, downsample) and StoreColor(QFloat4Canvas*).
    record(ref, outputs=...) takes the output arrays by name ("tc", "depth",
    "full", "half", "quads", and "full_mid", "quads_mid" when stores come
    between the draws); self.outputs holds host arrays of the right sizes."""

    def __init__(self, *a, color_depth=False, mid=False, **kw):
        super().__init__(*a, **kw)
        w, h = self.width, self.height
        self.color_depth = color_depth
        self.mid = mid
        self.outputs = {"tc": np.zeros(w * h, np.uint32), "full": np.zeros(w * h * 4, np.float32),
                        "half": np.zeros((w // 2) * (h // 2) * 4, np.float32),
                        "quads": np.zeros((w // 2) * (h // 2) * 16, np.float32)}
        if not color_depth:
            self.outputs["depth"] = np.zeros(w * h, np.float32)
        if mid:
            self.outputs["full_mid"] = np.zeros(w * h * 4, np.float32)
            self.outputs["quads_mid"] = np.zeros((w // 2) * (h // 2) * 16, np.float32)

    def record(self, ref=None, outputs=None, gamma=True, **_):
        gl = GL()
        ref = ref or (lambda k: self.arrays[k])
        out = outputs or self.outputs
        w, h = self.width, self.height
        self._record(gl, ref, out)
        gl.StoreColorFP(out["full"], w, h)
        gl.StoreColorFP(out["half"], w // 2, h // 2, downsample=True)
        gl.StoreColorQuads(out["quads"], w, h)
        gl.UseProgram(abi.PROGRAM_DEFAULT_POST)
        gl.StoreColor(out["tc"], w, h, gamma)
        if not self.color_depth:
            gl.StoreDepth(out["depth"])
        return gl


def float_store_frame(seed=21, ntris=6000, width=320, height=180, tile_blocks=(4, 4), color_depth=False, mid=False,
                      spread=0.35):
    """Random Gouraud triangles (the config-1 generator, shrunk by `spread`)
    drawn in two halves; the colour buffer is RB_RGBF32 with RB_F32 depth, or
    RB_COLOR_DEPTH (depth in the colour's w).  With mid=True the full float
    and quad stores are also taken between the two halves (stores between
    draws keep the raster pass in its sequential walk)."""
    base = plain_raster(seed=seed, ntris=ntris, width=width, height=height, tile_blocks=tile_blocks, spread=spread)
    arrays = base.arrays
    half = (ntris // 2) * 3

    def record(gl, ref, out):
        if color_depth:
            gl.RenderbufferType(abi.GL_COLOR_ATTACHMENT0, abi.RB_COLOR_DEPTH)
            gl.RenderbufferType(abi.GL_DEPTH_ATTACHMENT, abi.RB_COLOR_DEPTH)
            gl.ClearColor((0.05, 0.1, 0.15))
            gl.ClearDepth(1.0)
            gl.Clear(abi.GL_COLOR_BUFFER_BIT | abi.GL_DEPTH_BUFFER_BIT)
        else:
            _begin_frame(gl, (0.05, 0.1, 0.15))
        gl.UseProgram(abi.PROGRAM_GOURAUD)
        gl.UseBuffer(0, (ref("px"), ref("py"), ref("pz")))
        gl.UseBuffer(3, (ref("cr"), ref("cg"), ref("cb")))
        gl.DrawElements(half, ref("idx"), 0)
        if mid:
            gl.StoreColorFP(out["full_mid"], width, height)
            gl.StoreColorQuads(out["quads_mid"], width, height)
        gl.UseBuffer(0, tuple(ref(k)[half:] for k in ("px", "py", "pz")))
        gl.UseBuffer(3, tuple(ref(k)[half:] for k in ("cr", "cg", "cb")))
        gl.DrawElements(3 * ntris - half, ref("idx"), 0)

    name = "float_store_%s%s" % ("color_depth" if color_depth else "rgbf32", "_mid" if mid else "")
    return FloatStoreScene(name, width, height, tile_blocks, arrays, record, ntris, color_depth=color_depth, mid=mid)


def instanced_scene(seed=41, ninst=2000, width=640, height=360, tile_blocks=(4, 4), cull=True, near_share=0.004,
                    magic=0.625):
    """Instanced draws: ninst unit cubes drawn by one DrawElementsInstanced
    with ManyProgram (per-instance column-major mat4 in buffer 15: random
    rotation, size 0.3-0.8, centre in [-4,4]^2 x [-6,2]; a near_share of them
    around the near plane of the camera at (0,0,8), so some are clipped; uv
    per face corner; fragment colour (u, v, magic)), then 200 random Gouraud
    triangles drawn three times by one DrawArraysInstanced (instances of a
    program without instance data are copies).  Back faces culled for the
    cubes when `cull`."""
    pos, _, tri = _cube_mesh()
    uv = np.array([[(su + 1) / 2, (sv + 1) / 2] for _ in range(6) for (su, sv) in ((-1, -1), (1, -1), (1, 1), (-1, 1))])
    u = uniform01(seed * 131 + 7, ninst * 8).reshape(ninst, 8).astype(np.float64)
    rot = _random_rotations(u[:, 0:3])
    size = 0.3 + 0.5 * u[:, 3]
    centre = np.stack([-4 + 8 * u[:, 4], -4 + 8 * u[:, 5], -6 + 8 * u[:, 6]], 1)
    near = u[:, 7] < near_share
    centre[near] = np.stack([-1.5 + 3.0 * u[near, 4], -0.9 + 1.8 * u[near, 5], 7.4 + 1.2 * u[near, 6]], 1)
    m = np.zeros((ninst, 4, 4))
    m[:, :3, :3] = rot * size[:, None, None]
    m[:, :3, 3] = centre
    m[:, 3, 3] = 1.0
    imat = np.ascontiguousarray(m.transpose(0, 2, 1).reshape(-1), np.float32)   # column-major per instance
    gt = plain_raster(seed=seed + 1, ntris=200, width=width, height=height, tile_blocks=tile_blocks, spread=0.5)
    arrays = {"cx": pad4(pos[:, 0]), "cy": pad4(pos[:, 1]), "cz": pad4(pos[:, 2]),
              "cu": pad4(uv[:, 0]), "cv": pad4(uv[:, 1]), "cidx": np.ascontiguousarray(tri.reshape(-1), np.uint16),
              "imat": imat}
    for k in ("px", "py", "pz", "cr", "cg", "cb"):
        arrays["g" + k] = gt.arrays[k]
    view = look_at((0.0, 0.0, 8.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0))
    proj = perspective(60.0, width / height, 0.1, 100.0)
    ident = np.eye(4, dtype=np.float32)

    def record(gl, ref):
        _begin_frame(gl, (0.02, 0.03, 0.05))
        gl.UseProgram(abi.PROGRAM_MANY)
        gl.UseUniforms([magic])
        if cull:
            gl.Enable(abi.GL_CULL_FACE)
            gl.CullFace(abi.GL_BACK)
        gl.ViewMatrix(view)
        gl.ProjectionMatrix(proj)
        gl.UseBuffer(0, (ref("cx"), ref("cy"), ref("cz")))
        gl.UseBuffer(9, ref("cu"))
        gl.UseBuffer(10, ref("cv"))
        gl.UseBuffer(15, ref("imat"))
        gl.DrawElementsInstanced(len(tri) * 3, ref("cidx"), ninst)
        gl.Disable(abi.GL_CULL_FACE)
        gl.UseProgram(abi.PROGRAM_GOURAUD)
        gl.UseUniforms([0.0])
        gl.ViewMatrix(ident)
        gl.ProjectionMatrix(ident)
        gl.UseBuffer(0, (ref("gpx"), ref("gpy"), ref("gpz")))
        gl.UseBuffer(3, (ref("gcr"), ref("gcg"), ref("gcb")))
        gl.UseBuffer(9, None)
        gl.UseBuffer(10, None)
        gl.UseBuffer(15, None)
        gl.DrawArraysInstanced(3 * 200, 3)

    return Scene("instanced_%d" % ninst, width, height, tile_blocks, arrays, record, ninst * len(tri) + 600)


def obj1_scene(seed=51, nspheres=24, divs=3, width=640, height=360, tile_blocks=(4, 4), dense_hint=False):
    """OBJ1Program (src/viewer/shaders.hxx:586-699): icospheres (radius
    8-20, smooth normals, random per-vertex kd in [0.2, 1]) placed 60-260
    units in front of a camera at the origin looking down -z, so the
    program's point light at the eye gives diffuse * 100/distance mostly
    below 1; one sphere straddles the near plane (clipped).  Each sphere is
    one DrawElements (the 1P binning path, or with dense_hint the 2P path)."""
    verts, faces = icosphere(divs)
    nv = len(verts)
    u = uniform01(seed * 977 + 3, nspheres * 5).reshape(nspheres, 5).astype(np.float64)
    radius = 8.0 + 12.0 * u[:, 0]
    centre = np.stack([-60 + 120 * u[:, 1], -35 + 70 * u[:, 2], -(60 + 200 * u[:, 3])], 1)
    # sphere 0 reaches 0.74 units from the eye, closer than the near plane (1):
    # the plane cuts its visible cap, so front faces are clipped and kept
    centre[0] = (0.5, 0.3, -4.7)
    radius[0] = 4.0
    kd = 0.2 + 0.8 * uniform01(seed * 977 + 11, nspheres * nv * 3).reshape(nspheres, nv, 3)
    arrays = {"idx": np.ascontiguousarray(faces.reshape(-1), np.uint16)}
    for i in range(nspheres):
        p = verts * radius[i] + centre[i]
        arrays["p%d" % i] = np.ascontiguousarray(np.stack([pad4(p[:, 0]), pad4(p[:, 1]), pad4(p[:, 2])]))
        arrays["n%d" % i] = np.ascontiguousarray(np.stack([pad4(verts[:, 0]), pad4(verts[:, 1]), pad4(verts[:, 2])]))
        arrays["k%d" % i] = np.ascontiguousarray(np.stack([pad4(kd[i, :, 0]), pad4(kd[i, :, 1]), pad4(kd[i, :, 2])]))
    view = look_at((0.0, 0.0, 0.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0))
    proj = perspective(60.0, width / height, 1.0, 1000.0)
    hint = (abi.RGL_HINT_DENSE | abi.RGL_HINT_READ4) if dense_hint else 0

    def record(gl, ref):
        _begin_frame(gl, (0.0, 0.0, 0.0))
        gl.UseProgram(abi.PROGRAM_OBJ1)
        gl.Enable(abi.GL_CULL_FACE)
        gl.CullFace(abi.GL_BACK)
        gl.ViewMatrix(view)
        gl.ProjectionMatrix(proj)
        for i in range(nspheres):
            gl.UseBuffer(0, tuple(ref("p%d" % i)[k] for k in range(3)))
            gl.UseBuffer(3, tuple(ref("n%d" % i)[k] for k in range(3)))
            gl.UseBuffer(6, tuple(ref("k%d" % i)[k] for k in range(3)))
            gl.DrawElements(len(faces) * 3, ref("idx"), hint)

    return Scene("obj1_%d" % nspheres, width, height, tile_blocks, arrays, record, nspheres * len(faces))
