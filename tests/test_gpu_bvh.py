"""GPU binned-SAH BLAS builder against the host builder: every BVH it produces is structurally
valid (each triangle in exactly one leaf, child boxes equal to the union of their subtree's
triangle boxes, leaves of at most 4 triangles, depth within the traversal stack budget), its SAH
cost is close to the host builder's, and renders through either BVH are bit-identical (closest
hits keep the smallest (t, instance, triangle), so they do not depend on the tree)."""
import ctypes
import time

import numpy as np
import pytest

from aurora_gb300 import _abi

pytestmark = pytest.mark.gpu


def read_bvh(r, geom):
    lib = r._lib
    root, depth, nn = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_uint32()
    _abi.check(lib.agb_geometry_bvh(r.ctx, geom, None, 0, None, 0, ctypes.byref(root), ctypes.byref(depth),
                                    ctypes.byref(nn)))
    ntri = len(r.scene.meshes[geom]["indices"]) // 3
    nodes = np.zeros((max(nn.value, 1), 16), np.float32)
    tris = np.zeros((ntri, 12), np.float32)
    _abi.check(lib.agb_geometry_bvh(r.ctx, geom, nodes.ctypes.data, nodes.shape[0], tris.ctypes.data, ntri,
                                    None, None, None))
    return nodes[:nn.value], tris, root.value, depth.value


def check_and_cost(nodes, tris, root, depth, ntri):
    """Validates the tree; returns its SAH cost (node areas relative to the root box, interior 1,
    per-triangle 1)."""
    ids = tris[:, 3].view(np.int32)
    assert sorted(ids.tolist()) == list(range(ntri)), "triangle ids are not a permutation"
    v = tris.reshape(ntri, 3, 4)[:, :, :3]
    tlo, thi = v.min(axis=1), v.max(axis=1)
    refs = nodes[:, 12:14].view(np.int32) if len(nodes) else np.zeros((0, 2), np.int32)
    seen = np.zeros(ntri, np.int32)
    area = lambda lo, hi: 2.0 * float((hi - lo)[0] * (hi - lo)[1] + (hi - lo)[1] * (hi - lo)[2] + (hi - lo)[2] * (hi - lo)[0])
    cost = [0.0]
    max_depth = [0]

    def visit(ref, d):
        max_depth[0] = max(max_depth[0], d)
        if ref < 0:
            code = ~ref
            first, count = code >> 3, (code & 7) + 1
            assert count <= 4
            seen[first:first + count] += 1
            lo, hi = tlo[first:first + count].min(axis=0), thi[first:first + count].max(axis=0)
            return lo, hi, count
        n = nodes[ref]
        boxes = [(np.array([n[0], n[2], n[8]]), np.array([n[1], n[3], n[9]])),
                 (np.array([n[4], n[6], n[10]]), np.array([n[5], n[7], n[11]]))]
        out_lo, out_hi = np.full(3, np.inf, np.float32), np.full(3, -np.inf, np.float32)
        for side in (0, 1):
            lo, hi, count = visit(int(refs[ref][side]), d + 1)
            np.testing.assert_array_equal(boxes[side][0], lo)
            np.testing.assert_array_equal(boxes[side][1], hi)
            a = area(lo, hi)
            cost[0] += a * (count if int(refs[ref][side]) < 0 else 1.0)
            out_lo, out_hi = np.minimum(out_lo, lo), np.maximum(out_hi, hi)
        return out_lo, out_hi, 0

    lo, hi, _ = visit(root, 0)
    assert (seen == 1).all(), "a triangle is in zero or several leaves"
    assert max_depth[0] == depth and depth <= 34
    root_area = area(lo, hi)
    return cost[0] / root_area if root_area > 0 else 0.0


def meshes():
    from aurora_gb300 import scenes
    rng = np.random.default_rng(3)
    out = {"icosphere5": scenes.icosphere(5, radius=2.0, displacement=0.02, seed=1),
           "uv_sphere": scenes.uv_sphere(32, 16, 1.0)}
    p = rng.uniform(-5, 5, (3000, 3)).astype(np.float32)
    out["soup"] = (p + rng.normal(0, 0.2, p.shape).astype(np.float32), None, None,
                   np.arange(3000, dtype=np.uint32))
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    out["identical"] = (np.tile(tri, (200, 1)), None, None, np.arange(600, dtype=np.uint32))
    out["three_triangles"] = (rng.uniform(-1, 1, (9, 3)).astype(np.float32), None, None,
                              np.arange(9, dtype=np.uint32))
    return out


@pytest.mark.parametrize("name", ["icosphere5", "uv_sphere", "soup", "identical", "three_triangles"])
def test_gpu_bvh_valid_and_close_to_host(agb, name):
    from aurora_gb300 import api, scenes
    pos, nrm, uv, idx = meshes()[name]
    costs = {}
    for builder in (_abi.BVH_HOST, _abi.BVH_GPU):
        s = scenes.SceneDesc(name)
        s.add_mesh(pos, nrm, uv, idx)
        with api.Renderer() as r:
            _abi.check(r._lib.agb_set_bvh_builder(r.ctx, builder))
            r.upload_geometry_only(s)
            nodes, tris, root, depth = read_bvh(r, 0)
        costs[builder] = check_and_cost(nodes, tris, root, depth, len(idx) // 3)
    print(f"{name}: SAH cost host {costs[_abi.BVH_HOST]:.2f} gpu {costs[_abi.BVH_GPU]:.2f}")
    assert costs[_abi.BVH_GPU] <= 1.15 * costs[_abi.BVH_HOST] + 1e-6


@pytest.mark.parametrize("config", ["small", "large", "layered"])
def test_renders_identical_with_gpu_and_host_bvh(agb, config):
    from aurora_gb300 import api, scenes
    if config == "small":
        s = scenes.config_small(width=96, height=64, spp=4)
    elif config == "large":
        s = scenes.config_large(width=96, height=64, spp=4, level=6, instances=16, env_size=(64, 32))
    else:
        s = scenes.config_layered(width=64, height=48, spp=4, blas=2, instances=6, tri_range=(300, 900),
                                  decal_size=64)
    imgs = []
    for builder in (_abi.BVH_HOST, _abi.BVH_GPU):
        with api.Renderer() as r:
            _abi.check(r._lib.agb_set_bvh_builder(r.ctx, builder))
            r.upload(s)
            r.render(0, s.spp)
            imgs.append(r.read(_abi.ACCUM_RUNNING_MEAN))
    np.testing.assert_array_equal(imgs[0], imgs[1])


def test_gpu_bvh_build_time_1m_triangles(agb):
    """Icosphere level 8 (1,310,720 triangles): GPU build against the host build, and the tree's
    SAH cost against the host's."""
    from aurora_gb300 import api, scenes
    pos, nrm, uv, idx = scenes.icosphere(8, radius=6.0, displacement=0.02, seed=1)
    out = {}
    for builder in (_abi.BVH_HOST, _abi.BVH_GPU):
        s = scenes.SceneDesc("ico8")
        s.add_mesh(pos, nrm, uv, idx)
        with api.Renderer() as r:
            _abi.check(r._lib.agb_set_bvh_builder(r.ctx, builder))
            r.upload_geometry_only(s)     # warm the allocations
            t0 = time.perf_counter()
            r.upload_geometry_only(s)
            out[builder] = time.perf_counter() - t0
    print(f"1.31M-triangle BLAS: host {out[_abi.BVH_HOST] * 1e3:.0f} ms, gpu {out[_abi.BVH_GPU] * 1e3:.0f} ms "
          f"(both include the upload)")
    assert out[_abi.BVH_GPU] < out[_abi.BVH_HOST]


def read_tlas(r):
    lib = r._lib
    root, depth, nn = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_uint32()
    _abi.check(lib.agb_tlas_read(r.ctx, None, 0, None, 0, ctypes.byref(root), ctypes.byref(depth),
                                 ctypes.byref(nn)))
    n = len(r.scene.instances)
    nodes = np.zeros((max(nn.value, 1), 16), np.float32)
    order = np.zeros(n, np.int32)
    _abi.check(lib.agb_tlas_read(r.ctx, nodes.ctypes.data, nodes.shape[0], order.ctypes.data, n,
                                 None, None, None))
    return nodes[:nn.value], order, root.value, depth.value


def check_tlas(s, nodes, order, root, depth):
    """One instance per leaf, every instance in exactly one leaf, each leaf box containing its
    instance's world-space vertices, each interior box containing its children's, depth as
    reported."""
    n = len(s.instances)
    assert sorted(order.tolist()) == list(range(n))
    world = []
    for inst in s.instances:
        p = s.meshes[inst["mesh"]]["positions"].astype(np.float64)
        m = np.asarray(inst["xform"], np.float64).reshape(3, 4)
        w = p @ m[:, :3].T + m[:, 3]
        world.append((w.min(0), w.max(0)))
    refs = nodes[:, 12:14].view(np.int32) if len(nodes) else np.zeros((0, 2), np.int32)
    seen = np.zeros(n, np.int32)
    max_depth = [0]

    def visit(ref, d, lo_box, hi_box):
        max_depth[0] = max(max_depth[0], d)
        if ref < 0:
            code = ~ref
            slot, count = code >> 3, (code & 7) + 1
            assert count == 1
            inst = order[slot]
            seen[inst] += 1
            if lo_box is not None:
                lo, hi = world[inst]
                assert (lo_box <= lo + 1e-4 * (1 + np.abs(lo))).all() and \
                    (hi_box >= hi - 1e-4 * (1 + np.abs(hi))).all()
            return
        nd = nodes[ref]
        boxes = [(np.array([nd[0], nd[2], nd[8]]), np.array([nd[1], nd[3], nd[9]])),
                 (np.array([nd[4], nd[6], nd[10]]), np.array([nd[5], nd[7], nd[11]]))]
        for side in (0, 1):
            lo, hi = boxes[side]
            if lo_box is not None:
                assert (lo >= lo_box).all() and (hi <= hi_box).all()
            visit(int(refs[ref][side]), d + 1, lo, hi)

    visit(root, 0, None, None)
    assert (seen == 1).all()
    assert max_depth[0] == depth


@pytest.mark.parametrize("instances", [1, 2, 1000, 5000])
def test_tlas_gpu_and_host_valid_and_render_identically(agb, oracle, instances):
    """TLAS over many instances built by the GPU builder (the BLAS kernel over instance boxes) and
    by the host builder: both valid; renders through either identical to each other and to the
    oracle; 5000 instances need more than the former fixed 12-level TLAS budget."""
    from aurora_gb300 import api, scenes
    s = scenes.config_stress(width=64, height=48, spp=2, blas=3, instances=instances,
                             tri_range=(200, 2000), decal_size=64, box=60.0 if instances > 2 else 6.0)
    imgs, depths = [], []
    for builder in (_abi.BVH_HOST, _abi.BVH_GPU):
        with api.Renderer() as r:
            _abi.check(r._lib.agb_set_bvh_builder(r.ctx, builder))
            r.upload(s)
            nodes, order, root, depth = read_tlas(r)
            check_tlas(s, nodes, order, root, depth)
            depths.append(depth)
            r.render(0, s.spp)
            imgs.append(r.read(_abi.ACCUM_RUNNING_MEAN))
    o = oracle.OracleScene(s).render(0, s.spp)["mean"]
    print(f"{instances} instances: TLAS depth host {depths[0]} gpu {depths[1]}; relMSE vs oracle "
          f"{oracle.rel_mse(imgs[1], o):.3g}")
    np.testing.assert_array_equal(imgs[0], imgs[1])
    assert oracle.rel_mse(imgs[1], o) < 1e-9
    if instances == 5000:
        assert depths[1] > 12
