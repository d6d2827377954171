"""The seeded synthetic inputs of the build and traversal benchmarks
(clear_gb300/workloads.py) have the stated shapes and distributions:
centroids uniform in [0,1]^3 with vertex offsets of mean 0.5 n^(-1/3) along
uniform directions, closest-hit origins uniform in [-0.1,1.1]^3 with unit
directions and infinite tmax, shadow segments between points of [0,1]^3 with
their length as tmax; and they are reproducible from their seeds."""
import numpy as np

from clear_gb300 import workloads as W


def test_triangle_soup_layout_and_distribution():
    n = 1 << 16
    vx, vy, vz = W.triangle_soup(n, seed=11)
    assert all(a.dtype == np.float32 and a.shape == (3 * n,) and a.flags.c_contiguous for a in (vx, vy, vz))
    v = np.stack([vx, vy, vz], axis=1).astype(np.float64).reshape(n, 3, 3)
    # the centroid is not stored; the vertex mean is the centroid plus the
    # mean offset, whose spread is small next to the unit cube
    mean = v.mean(axis=1)
    assert np.all(mean > -0.2) and np.all(mean < 1.2)
    assert abs(mean.mean() - 0.5) < 0.01 and abs(mean.std() - np.sqrt(1 / 12)) < 0.01
    # edge length ~ Exp(mean 0.5 n^(-1/3)) per vertex: the mean vertex-to-vertex
    # distance sits on that scale
    scale = 0.5 * n ** (-1.0 / 3.0)
    edge = np.linalg.norm(v[:, 1] - v[:, 0], axis=1)
    assert 0.8 * scale < np.median(edge) < 2.0 * scale
    a, b, c = W.triangle_soup(n, seed=11)
    assert np.array_equal(a, vx) and np.array_equal(b, vy) and np.array_equal(c, vz)
    assert not np.array_equal(W.triangle_soup(n, seed=12)[0], vx)


def test_closest_rays_layout_and_distribution():
    m = 1 << 16
    r = W.closest_rays(m, seed=4)
    assert r.dtype == np.float32 and r.shape == (m, 8)
    o, d = r[:, 0:3], r[:, 4:7].astype(np.float64)
    assert o.min() >= -0.1 and o.max() <= 1.1 and abs(o.mean() - 0.5) < 0.01
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
    assert np.all(np.abs(d.mean(axis=0)) < 0.02)  # uniform on the sphere
    assert np.all(np.isinf(r[:, 3])) and np.all(r[:, 7] == 0)
    assert np.array_equal(W.closest_rays(m, seed=4), r)


def test_shadow_rays_are_segments_inside_the_cube():
    m = 1 << 14
    r = W.shadow_rays(m, seed=5)
    o, d, L = r[:, 0:3].astype(np.float64), r[:, 4:7].astype(np.float64), r[:, 3].astype(np.float64)
    assert o.min() >= 0 and o.max() <= 1
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
    end = o + d * L[:, None]
    assert end.min() > -1e-5 and end.max() < 1 + 1e-5
    assert np.all(L > 0) and L.max() <= np.sqrt(3) + 1e-6
