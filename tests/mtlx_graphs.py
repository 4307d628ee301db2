"""MaterialX node-graph test documents and helpers: decoding the `materialx_graph` property (the
compiled program), a numpy interpreter of its operations (the semantics include/agb.h documents
for agb_material_graphs_set), and attaching programs to a SceneDesc."""
import numpy as np

from aurora_gb300 import _abi

# A custom node (nodedef + implementing nodegraph) making a checker from texture coordinates, mixed
# into base_color; specular_roughness from the object-space position through sin and clamp.
CHECKER = """<?xml version="1.0"?>
<materialx version="1.39" colorspace="lin_rec709">
  <nodedef name="ND_tiles_float" node="tiles">
    <input name="count" type="vector2" value="4.0, 4.0" />
    <output name="out" type="float" />
  </nodedef>
  <nodegraph name="NG_tiles_float" nodedef="ND_tiles_float">
    <texcoord name="uv" type="vector2" />
    <multiply name="scaled" type="vector2">
      <input name="in1" type="vector2" nodename="uv" />
      <input name="in2" type="vector2" interfacename="count" />
    </multiply>
    <floor name="cell" type="vector2">
      <input name="in" type="vector2" nodename="scaled" />
    </floor>
    <extract name="cx" type="float">
      <input name="in" type="vector2" nodename="cell" />
      <input name="index" type="integer" value="0" />
    </extract>
    <extract name="cy" type="float">
      <input name="in" type="vector2" nodename="cell" />
      <input name="index" type="integer" value="1" />
    </extract>
    <add name="sum" type="float">
      <input name="in1" type="float" nodename="cx" />
      <input name="in2" type="float" nodename="cy" />
    </add>
    <modulo name="parity" type="float">
      <input name="in1" type="float" nodename="sum" />
      <input name="in2" type="float" value="2.0" />
    </modulo>
    <output name="out" type="float" nodename="parity" />
  </nodegraph>
  <tiles name="pattern" type="float">
    <input name="count" type="vector2" value="8.0, 6.0" />
  </tiles>
  <mix name="tinted" type="color3">
    <input name="fg" type="color3" value="0.8, 0.2, 0.1" />
    <input name="bg" type="color3" value="0.1, 0.3, 0.7" />
    <input name="mix" type="float" nodename="pattern" />
  </mix>
  <position name="pos" type="vector3" />
  <extract name="px" type="float">
    <input name="in" type="vector3" nodename="pos" />
    <input name="index" type="integer" value="0" />
  </extract>
  <multiply name="px3" type="float">
    <input name="in1" type="float" nodename="px" />
    <input name="in2" type="float" value="3.0" />
  </multiply>
  <sin name="wave" type="float">
    <input name="in" type="float" nodename="px3" />
  </sin>
  <clamp name="rough" type="float">
    <input name="in" type="float" nodename="wave" />
    <input name="low" type="float" value="0.15" />
    <input name="high" type="float" value="0.8" />
  </clamp>
  <standard_surface name="sr" type="surfaceshader">
    <input name="base_color" type="color3" nodename="tinted" />
    <input name="specular_roughness" type="float" nodename="rough" />
    <input name="metalness" type="float" value="0.3" />
  </standard_surface>
  <surfacematerial name="m" type="material">
    <input name="surfaceshader" type="surfaceshader" nodename="sr" />
  </surfacematerial>
</materialx>
"""

# A node graph with its own interface input, an image sampled through tiled texture coordinates
# (base_color and, through luminance / ifgreater, the emission), a normal map built from the
# texture coordinates, coat roughness from a switch over the world-space normal, and an opacity
# from a swizzle and power.
PATTERNS = """<?xml version="1.0"?>
<materialx version="1.39" colorspace="lin_rec709">
  <nodegraph name="NG">
    <input name="tint" type="color3" value="0.9, 0.8, 0.6" />
    <texcoord name="uv" type="vector2" />
    <multiply name="uv2" type="vector2">
      <input name="in1" type="vector2" nodename="uv" />
      <input name="in2" type="float" value="3.0" />
    </multiply>
    <image name="tex" type="color3">
      <input name="file" type="filename" value="pattern.png" />
      <input name="texcoord" type="vector2" nodename="uv2" />
    </image>
    <multiply name="tinted" type="color3">
      <input name="in1" type="color3" nodename="tex" />
      <input name="in2" type="color3" interfacename="tint" />
    </multiply>
    <luminance name="lum" type="color3">
      <input name="in" type="color3" nodename="tex" />
    </luminance>
    <extract name="l" type="float">
      <input name="in" type="color3" nodename="lum" />
      <input name="index" type="integer" value="0" />
    </extract>
    <ifgreater name="glow" type="color3">
      <input name="value1" type="float" nodename="l" />
      <input name="value2" type="float" value="0.6" />
      <input name="in1" type="color3" value="1.0, 0.5, 0.2" />
      <input name="in2" type="color3" value="0, 0, 0" />
    </ifgreater>
    <extract name="u" type="float">
      <input name="in" type="vector2" nodename="uv" />
      <input name="index" type="integer" value="0" />
    </extract>
    <multiply name="u8" type="float">
      <input name="in1" type="float" nodename="u" />
      <input name="in2" type="float" value="25.0" />
    </multiply>
    <sin name="su" type="float">
      <input name="in" type="float" nodename="u8" />
    </sin>
    <cos name="cu" type="float">
      <input name="in" type="float" nodename="u8" />
    </cos>
    <remap name="nx" type="float">
      <input name="in" type="float" nodename="su" />
      <input name="inlow" type="float" value="-1" />
      <input name="inhigh" type="float" value="1" />
    </remap>
    <remap name="ny" type="float">
      <input name="in" type="float" nodename="cu" />
      <input name="inlow" type="float" value="-1" />
      <input name="inhigh" type="float" value="1" />
    </remap>
    <combine3 name="nmap" type="vector3">
      <input name="in1" type="float" nodename="nx" />
      <input name="in2" type="float" nodename="ny" />
      <input name="in3" type="float" value="1.0" />
    </combine3>
    <normalmap name="bump" type="vector3">
      <input name="in" type="vector3" nodename="nmap" />
      <input name="scale" type="float" value="0.6" />
    </normalmap>
    <normal name="nw" type="vector3">
      <input name="space" type="string" value="world" />
    </normal>
    <dotproduct name="up" type="float">
      <input name="in1" type="vector3" nodename="nw" />
      <input name="in2" type="vector3" value="0, 1, 0" />
    </dotproduct>
    <add name="which" type="float">
      <input name="in1" type="float" nodename="up" />
      <input name="in2" type="float" value="1.0" />
    </add>
    <switch name="cr" type="float">
      <input name="in1" type="float" value="0.9" />
      <input name="in2" type="float" value="0.3" />
      <input name="in3" type="float" value="0.05" />
      <input name="which" type="float" nodename="which" />
    </switch>
    <swizzle name="rr" type="color3">
      <input name="in" type="color3" nodename="tex" />
      <input name="channels" type="string" value="ggb" />
    </swizzle>
    <power name="op" type="color3">
      <input name="in1" type="color3" nodename="rr" />
      <input name="in2" type="float" value="0.25" />
    </power>
    <output name="base" type="color3" nodename="tinted" />
    <output name="emit" type="color3" nodename="glow" />
    <output name="n" type="vector3" nodename="bump" />
    <output name="coatr" type="float" nodename="cr" />
    <output name="opac" type="color3" nodename="op" />
  </nodegraph>
  <standard_surface name="sr" type="surfaceshader">
    <input name="base_color" type="color3" nodegraph="NG" output="base" />
    <input name="emission" type="float" value="1.0" />
    <input name="emission_color" type="color3" nodegraph="NG" output="emit" />
    <input name="normal" type="vector3" nodegraph="NG" output="n" />
    <input name="coat" type="float" value="0.6" />
    <input name="coat_roughness" type="float" nodegraph="NG" output="coatr" />
    <input name="opacity" type="color3" nodegraph="NG" output="opac" />
  </standard_surface>
</materialx>
"""


# Noise nodes: base_color mixed by a three-octave fractal of the object-space position,
# specular_roughness from 2D Perlin noise of the scaled texcoord, emission from 3D cell noise.
NOISE = """<?xml version="1.0"?>
<materialx version="1.39">
  <position name="p" type="vector3" />
  <multiply name="p4" type="vector3">
    <input name="in1" type="vector3" nodename="p" />
    <input name="in2" type="float" value="4.0" />
  </multiply>
  <fractal3d name="marble" type="float">
    <input name="position" type="vector3" nodename="p4" />
    <input name="amplitude" type="float" value="0.8" />
    <input name="octaves" type="integer" value="3" />
    <input name="lacunarity" type="float" value="2.1" />
    <input name="diminish" type="float" value="0.45" />
  </fractal3d>
  <add name="marble01" type="float">
    <input name="in1" type="float" nodename="marble" />
    <input name="in2" type="float" value="0.5" />
  </add>
  <mix name="veins" type="color3">
    <input name="fg" type="color3" value="0.9, 0.85, 0.8" />
    <input name="bg" type="color3" value="0.15, 0.2, 0.3" />
    <input name="mix" type="float" nodename="marble01" />
  </mix>
  <texcoord name="uv" type="vector2" />
  <multiply name="uv8" type="vector2">
    <input name="in1" type="vector2" nodename="uv" />
    <input name="in2" type="float" value="8.0" />
  </multiply>
  <noise2d name="grain" type="float">
    <input name="texcoord" type="vector2" nodename="uv8" />
    <input name="amplitude" type="float" value="0.3" />
    <input name="pivot" type="float" value="0.45" />
  </noise2d>
  <cellnoise3d name="cells" type="float">
    <input name="position" type="vector3" nodename="p4" />
  </cellnoise3d>
  <multiply name="glow" type="color3">
    <input name="in1" type="color3" value="0.6, 0.3, 0.1" />
    <input name="in2" type="float" nodename="cells" />
  </multiply>
  <standard_surface name="S" type="surfaceshader">
    <input name="base_color" type="color3" nodename="veins" />
    <input name="specular_roughness" type="float" nodename="grain" />
    <input name="emission_color" type="color3" nodename="glow" />
    <input name="emission" type="float" value="0.5" />
  </standard_surface>
</materialx>
"""


def decode(program):
    """The `materialx_graph` strings -> (ops GRAPH_OP_DTYPE, consts float32 (K, 4), image paths)."""
    ops, consts, images = [], [], []
    for line in program:
        kind, rest = line.split(" ", 1)
        if kind == "op":
            ops.append(tuple(int(v) for v in rest.split()))
        elif kind == "const":
            consts.append([float(v) for v in rest.split()])
        elif kind == "image":
            images.append(rest)
    return (np.array(ops, _abi.GRAPH_OP_DTYPE), np.array(consts, np.float32).reshape(-1, 4), images)


def attach(s, programs):
    """programs: {material index: (ops, consts, scene image index per program image)} -> s.graphs."""
    n = len(s.materials)
    first = np.zeros(n, np.int32)
    count = np.zeros(n, np.int32)
    all_ops, all_k = [], []
    nk = 0
    for m in sorted(programs):
        ops, consts, image_map = programs[m]
        ops = ops.copy()
        isk = ops["op"] == _abi.GOP_CONST
        ops["imm"][isk] += nk
        isi = ops["op"] == _abi.GOP_IMAGE
        ops["imm"][isi] = np.asarray(image_map, np.uint16)[ops["imm"][isi]] if isi.any() else 0
        first[m] = sum(len(o) for o in all_ops)
        count[m] = len(ops)
        all_ops.append(ops)
        all_k.append(consts)
        nk += len(consts)
    s.graphs = dict(first=first, count=count, ops=np.concatenate(all_ops),
                    consts=np.concatenate(all_k).reshape(-1, 4))


# MaterialX's noise functions (its stdlib mx_noise.glsl, after OSL) in float32 numpy: lookup3's
# final mix as the lattice hash, improved-noise gradients and fade, 0.6616 / 0.9820 scales.
def _rotl(x, k):
    return (x << np.uint32(k)) | (x >> np.uint32(32 - k))


def _final(a, b, c):
    c = (c ^ b) - _rotl(b, 14)
    a = (a ^ c) - _rotl(c, 11)
    b = (b ^ a) - _rotl(a, 25)
    c = (c ^ b) - _rotl(b, 16)
    a = (a ^ c) - _rotl(c, 4)
    b = (b ^ a) - _rotl(a, 14)
    c = (c ^ b) - _rotl(b, 24)
    return c


def noise_hash(*cells):
    """lookup3-style hash of integer lattice coordinates (int arrays), as MaterialX seeds it."""
    seed = np.uint32((0xdeadbeef + (len(cells) << 2) + 13) & 0xffffffff)
    v = [seed + np.asarray(c).astype(np.int64).astype(np.uint32) for c in cells] + [seed] * (3 - len(cells))
    with np.errstate(over="ignore"):
        return _final(*[np.asarray(x, np.uint32) for x in v])


def _fade(t):
    f = np.float32
    return t * t * t * (t * (t * f(6) - f(15)) + f(10))


def _neg(v, n):
    return np.where(n != 0, -v, v)


def perlin2(x, y):
    f = np.float32
    X, Y = np.floor(x), np.floor(y)
    fx, fy = (x - X).astype(f), (y - Y).astype(f)
    X, Y = X.astype(np.int64), Y.astype(np.int64)

    def g(h, a, b):
        h = h & np.uint32(7)
        lo = h < 4
        u, v = np.where(lo, a, b), f(2) * np.where(lo, b, a)
        return _neg(u, h & np.uint32(1)) + _neg(v, h & np.uint32(2))
    u, v = _fade(fx), _fade(fy)
    g0 = g(noise_hash(X, Y), fx, fy)
    g1 = g(noise_hash(X + 1, Y), fx - f(1), fy)
    g2 = g(noise_hash(X, Y + 1), fx, fy - f(1))
    g3 = g(noise_hash(X + 1, Y + 1), fx - f(1), fy - f(1))
    s1, t1 = f(1) - u, f(1) - v
    return (f(0.6616) * (t1 * (g0 * s1 + g1 * u) + v * (g2 * s1 + g3 * u))).astype(f)


def perlin3(x, y, z):
    f = np.float32
    X, Y, Z = np.floor(x), np.floor(y), np.floor(z)
    fx, fy, fz = (x - X).astype(f), (y - Y).astype(f), (z - Z).astype(f)
    X, Y, Z = X.astype(np.int64), Y.astype(np.int64), Z.astype(np.int64)

    def g(h, a, b, c):
        h = h & np.uint32(15)
        u = np.where(h < 8, a, b)
        v = np.where(h < 4, b, np.where((h == 12) | (h == 14), a, c))
        return _neg(u, h & np.uint32(1)) + _neg(v, h & np.uint32(2))
    gs = []
    for k in range(8):
        dx, dy, dz = k & 1, (k >> 1) & 1, k >> 2
        gs.append(g(noise_hash(X + dx, Y + dy, Z + dz), fx - f(dx), fy - f(dy), fz - f(dz)))
    u, v, w = _fade(fx), _fade(fy), _fade(fz)
    s1, t1, r1 = f(1) - u, f(1) - v, f(1) - w
    return (f(0.9820) * (r1 * (t1 * (gs[0] * s1 + gs[1] * u) + v * (gs[2] * s1 + gs[3] * u)) +
                         w * (t1 * (gs[4] * s1 + gs[5] * u) + v * (gs[6] * s1 + gs[7] * u)))).astype(f)


def cell2(x, y):
    h = noise_hash(np.floor(x).astype(np.int64), np.floor(y).astype(np.int64))
    return h.astype(np.float32) / np.float32(0xffffffff)


def cell3(x, y, z):
    h = noise_hash(np.floor(x).astype(np.int64), np.floor(y).astype(np.int64), np.floor(z).astype(np.int64))
    return h.astype(np.float32) / np.float32(0xffffffff)


def evaluate(ops, consts, inputs, images=()):
    """Runs a program (float32, numpy) over arrays of hit attributes: inputs[k] = (P, 3) per
    GIN_* code (texcoord as (P, 2)); images: RGBA float32 arrays sampled nearest with repeat.
    Returns {GOUT_* code: (P, 3)}."""
    f32 = np.float32
    P = len(next(iter(inputs.values())))
    r = np.zeros((_abi.GRAPH_REGS, P, 4), f32)
    out = {}
    for o in ops:
        A, B, C, D = r[o["a"]], r[o["b"]], r[o["c"]], r[o["d"]]
        op, imm = int(o["op"]), int(o["imm"])
        with np.errstate(all="ignore"):
            if op == _abi.GOP_CONST:
                v = np.broadcast_to(consts[imm], (P, 4)).astype(f32)
            elif op == _abi.GOP_INPUT:
                q = np.asarray(inputs[imm], f32)
                v = np.zeros((P, 4), f32)
                v[:, :q.shape[1]] = q
            elif op in (_abi.GOP_ADD, _abi.GOP_SUB, _abi.GOP_MUL, _abi.GOP_DIV, _abi.GOP_MIN, _abi.GOP_MAX,
                        _abi.GOP_POW, _abi.GOP_MOD):
                v = {_abi.GOP_ADD: A + B, _abi.GOP_SUB: A - B, _abi.GOP_MUL: A * B, _abi.GOP_DIV: A / B,
                     _abi.GOP_MIN: np.fmin(A, B), _abi.GOP_MAX: np.fmax(A, B), _abi.GOP_POW: np.power(A, B),
                     _abi.GOP_MOD: A - B * np.floor(A / B)}[op]
            elif op in (_abi.GOP_FLOOR, _abi.GOP_CEIL, _abi.GOP_ABS, _abi.GOP_SIN, _abi.GOP_COS, _abi.GOP_SQRT,
                        _abi.GOP_SIGN):
                v = {_abi.GOP_FLOOR: np.floor, _abi.GOP_CEIL: np.ceil, _abi.GOP_ABS: np.abs, _abi.GOP_SIN: np.sin,
                     _abi.GOP_COS: np.cos, _abi.GOP_SQRT: np.sqrt, _abi.GOP_SIGN: np.sign}[op](A)
            elif op == _abi.GOP_CLAMP:
                v = np.fmin(np.fmax(A, B), C)
            elif op == _abi.GOP_MIX:
                v = B + C * (A - B)
            elif op in (_abi.GOP_DOT, _abi.GOP_NORMALIZE, _abi.GOP_LENGTH):
                d = int(o["d"])
                bb = B if op == _abi.GOP_DOT else A
                s = A[:, 0] * bb[:, 0]
                for c in range(1, d):
                    s = s + A[:, c] * bb[:, c]
                if op == _abi.GOP_DOT:
                    v = np.repeat(s[:, None], 4, 1)
                elif op == _abi.GOP_LENGTH:
                    v = np.repeat(np.sqrt(s)[:, None], 4, 1)
                else:
                    v = np.zeros((P, 4), f32)
                    v[:, :d] = A[:, :d] / np.sqrt(s)[:, None]
            elif op == _abi.GOP_SWIZZLE:
                v = A[:, [imm & 3, (imm >> 2) & 3, (imm >> 4) & 3, (imm >> 6) & 3]]
            elif op == _abi.GOP_COMBINE:
                v = np.stack([A[:, 0], B[:, 0], C[:, 0], D[:, 0]], 1)
            elif op == _abi.GOP_SELECT:
                t = {0: A[:, 0] > B[:, 0], 1: A[:, 0] >= B[:, 0], 2: A[:, 0] == B[:, 0]}[imm]
                v = np.where(t[:, None], C, D)
            elif op == _abi.GOP_IMAGE:
                im = images[imm]
                h, w = im.shape[:2]
                x = np.floor(A[:, 0] * w).astype(np.int64) % w
                y = np.floor(A[:, 1] * h).astype(np.int64) % h
                v = im[y, x].astype(f32)
            elif op == _abi.GOP_NORMALMAP:
                n_, t_ = (np.asarray(inputs[_abi.GIN_NORMAL_WORLD], f32), np.asarray(inputs[_abi.GIN_TANGENT_WORLD], f32))
                vv = A[:, :3] * f32(2) - f32(1)
                vv[:, :2] *= B[:, :1]
                bn = np.cross(n_, t_)
                bn /= np.linalg.norm(bn, axis=1, keepdims=True)
                n2 = t_ * vv[:, :1] + bn * vv[:, 1:2] + n_ * vv[:, 2:3]
                v = np.zeros((P, 4), f32)
                v[:, :3] = n2 / np.linalg.norm(n2, axis=1, keepdims=True)
            elif op == _abi.GOP_NOISE:
                q = (perlin2(A[:, 0], A[:, 1]) if imm == 0 else perlin3(A[:, 0], A[:, 1], A[:, 2]) if imm == 1
                     else cell2(A[:, 0], A[:, 1]) if imm == 2 else cell3(A[:, 0], A[:, 1], A[:, 2]))
                v = np.repeat(q[:, None], 4, 1)
            elif op == _abi.GOP_OUTPUT:
                out[imm] = A[:, :3].copy()
                continue
            else:
                raise ValueError(f"operation {op}")
        r[o["dst"]] = np.asarray(v, f32)
    return out
