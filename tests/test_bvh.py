"""Structure of the BVH the builder emits, in the reference StacklessBVHNode
layout (common/stackless_bvh.hpp:264-341), and closest-hit distances of the
oracle traversal against brute force."""
import numpy as np
import pytest

from raccoongpurender_gb300 import scenes
from tests.helpers import build


def _check_tree(sm, mesh, leaf):
    nodes, ids = sm.export_stackless()
    info = sm.info()
    assert info.depth <= 63
    assert sorted(ids.tolist()) == list(range(mesh.ntris))
    P = mesh.points
    tri = P[mesh.indices]  # (m, 3, 3)
    lo, hi = tri.min(1), tri.max(1)
    n = nodes.shape[0]
    seen = np.zeros(n, bool)
    stack = [(0, None)]
    while stack:
        i, parent = stack.pop()
        assert not seen[i]
        seen[i] = True
        nd = nodes[i]
        if parent is not None:
            assert nd["link_parent"] == parent
        if nd["primitive_indices_end"] == 0:  # branch
            L, R = int(nd["link_L"]), int(nd["link_R"])
            assert nodes[L]["link_sibling"] == R and nodes[R]["link_sibling"] == L
            assert L == i + 1  # pre-order numbering, left subtree first
            for c, blo, bhi in ((L, nd["L_lower"], nd["L_upper"]), (R, nd["R_lower"], nd["R_upper"])):
                # every primitive below c lies inside the child box
                sub = [c]
                prims = []
                while sub:
                    k = sub.pop()
                    if nodes[k]["primitive_indices_end"] == 0:
                        sub += [int(nodes[k]["link_L"]), int(nodes[k]["link_R"])]
                    else:
                        prims += ids[nodes[k]["primitive_indices_beg"]:nodes[k]["primitive_indices_end"]].tolist()
                assert (lo[prims] >= blo[:3]).all() and (hi[prims] <= bhi[:3]).all()
            stack += [(R, i), (L, i)]
        else:
            cnt = nd["primitive_indices_end"] - nd["primitive_indices_beg"]
            assert 1 <= cnt <= leaf
    assert seen.all()


@pytest.mark.parametrize("leaf", [1, 2, 4, 8])
def test_tree_structure(rg, po, leaf):
    mesh = scenes.displaced_icosphere(3, seed=7)
    mesh.materials = [rg.materials.lambertian()] * mesh.ntris
    sm, _ = build(mesh, leaf=leaf)
    _check_tree(sm, mesh, leaf)


def test_deterministic_build(rg):
    mesh = scenes.displaced_icosphere(5, seed=7)
    mesh.materials = [rg.materials.lambertian()] * mesh.ntris
    a = rg.SceneManager()
    a.addMesh(mesh)
    a.buildBVH(num_threads=1)
    b = rg.SceneManager()
    b.addMesh(mesh)
    b.buildBVH(num_threads=8)
    na, ia = a.export_stackless()
    nb, ib = b.export_stackless()
    assert na.tobytes() == nb.tobytes() and ia.tobytes() == ib.tobytes()


def brute_force_t(mesh, rays):
    """Moller-Trumbore in float64 for every ray against every triangle."""
    P = mesh.points.astype(np.float64)
    v0, v1, v2 = (P[mesh.indices[:, k]] for k in range(3))
    e1, e2 = v1 - v0, v2 - v0
    best = np.full(len(rays), np.inf)
    for i in range(len(rays)):
        o = rays.o[i].astype(np.float64)
        d = rays.d[i].astype(np.float64)
        p = np.cross(d, e2)
        det = (e1 * p).sum(1)
        ok = np.abs(det) > 1e-12
        inv = np.where(ok, 1.0 / np.where(ok, det, 1.0), 0.0)
        tv = o - v0
        u = (tv * p).sum(1) * inv
        q = np.cross(tv, e1)
        v = (d[None, :] * q).sum(1) * inv
        t = (e2 * q).sum(1) * inv
        hit = ok & (u >= 0) & (v >= 0) & (u + v <= 1) & (t >= 0)
        if hit.any():
            best[i] = t[hit].min()
    return best


def test_traversal_matches_brute_force(rg, po):
    mesh = scenes.displaced_icosphere(3, seed=7)
    mesh.materials = [rg.materials.lambertian()] * mesh.ntris
    sm, osc = build(mesh)
    prim, rnd = scenes.closest_hit_rays(mesh, res=24, n_random=400, seed=2)
    for rays in (prim, rnd):
        p, t, _ = osc.trace(rays.packed8())
        ref = brute_force_t(mesh, rays)
        hit = np.isfinite(ref)
        assert (p >= 0).sum() == hit.sum()
        np.testing.assert_allclose(t[hit], ref[hit], rtol=1e-5, atol=1e-6)


def test_oracle_builder_tree_and_hits(po):
    """The oracle's own tree (binned SAH flattened as create_stackless_bvh does,
    the reference arm's tree): preorder numbering with sibling and parent
    links, every triangle in exactly one leaf of at most 4, child boxes that
    hold their primitives, and closest hits equal to those on the product's
    tree (the oracle traversal on both)."""
    mesh = scenes.displaced_icosphere(5, seed=7)
    osc = po.OracleScene.from_mesh(mesh.points, mesh.indices, max_leaf=4, threads=4)
    nodes = osc.nodes.view(np.float32).reshape(-1, 24)
    links = osc.nodes.reshape(-1, 24)
    parent, L, R, sib, beg, end = (links[:, 16 + k] for k in range(6))
    n = links.shape[0]
    tri = mesh.points[mesh.indices]
    lo, hi = tri.min(1), tri.max(1)
    assert parent[0] == 0 and sib[0] == 0
    leaves = end > 0
    assert (end[leaves] - beg[leaves] <= 4).all()
    assert sorted(osc.prim_ids.tolist()) == list(range(mesh.ntris))
    for i in np.nonzero(~leaves)[0]:
        l, r = int(L[i]), int(R[i])
        assert l == i + 1 and parent[l] == i and parent[r] == i and sib[l] == r and sib[r] == l
    for i in np.nonzero(leaves)[0]:
        p = int(parent[i])
        box = (nodes[p, 0:3], nodes[p, 4:7]) if int(L[p]) == i else (nodes[p, 8:11], nodes[p, 12:15])
        ids = osc.prim_ids[beg[i]:end[i]]
        assert (lo[ids] >= box[0]).all() and (hi[ids] <= box[1]).all()
    assert n == 2 * leaves.sum() - 1
    sm, prod = build(mesh)
    co, inc = scenes.closest_hit_rays(mesh, res=96, n_random=20000, seed=3)
    for rays in (co, inc):
        a = osc.trace(rays.packed8(), threads=4, normals=False)
        b = prod.trace(rays.packed8(), threads=4, normals=False)
        assert (a[0] == b[0]).all() and (a[1].view(np.uint32) == b[1].view(np.uint32)).all()
