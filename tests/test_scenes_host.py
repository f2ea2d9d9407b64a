"""The seeded synthetic workloads (lbvh_gb300/scenes.py) on the host: the
same seed gives the same bytes on every call and in every order of calls,
and each generator keeps the shape, count and range its workload states."""
import numpy as np

from lbvh_gb300 import scenes


def test_uniform_is_counter_based():
    a = scenes.uniform(7, 3, 200_000)
    assert a.dtype == np.float64 and a.min() >= 0.0 and a.max() < 1.0
    # element i depends only on (seed, stream, i): any window reproduces it
    assert np.array_equal(scenes.uniform(7, 3, 1000, start=70_000), a[70_000:71_000])
    assert np.array_equal(scenes.uniform(7, 3, 1, start=199_999), a[-1:])
    assert not np.array_equal(scenes.uniform(7, 4, 1000), a[:1000])  # another stream
    assert abs(a.mean() - 0.5) < 0.01
    n = scenes.normal(7, 3, 200_000)
    assert abs(n.mean()) < 0.02 and abs(n.std() - 1.0) < 0.02


def test_generators_are_deterministic():
    for make in (lambda: scenes.soup(5000, 3), lambda: scenes.torus_scene(seed=11),
                 lambda: scenes.pinhole_rays(64, 32), lambda: scenes.incoherent_rays(scenes.soup(100, 1), 777, 5)):
        x, y = make(), make()
        assert x.dtype == np.float32 and x.tobytes() == y.tobytes()


def test_shapes_and_counts():
    assert scenes.soup(1234, 2).shape == (1234, 12)
    assert scenes.torus_scene(seed=11).shape == (8320, 12)  # 6,320-triangle torus + 2,000-triangle plane
    r = scenes.pinhole_rays(64, 32)
    assert r.shape == (64 * 32, 8)
    assert np.all(r[:, 6] == 0.0) and np.all(np.isinf(r[:, 7]))  # tmin 0, tmax +inf
    c = scenes.log_uniform_counts(4096, 64, 65536, 3)
    assert c.min() >= 64 and c.max() <= 65536
    assert scenes.example_spheres().shape == (3, 4)
    cam = scenes.example_camera_rays(8, 4).reshape(-1, 8)
    assert np.all(cam[:, 2] == 5.0) and np.all(cam[:, 5] == -1.0)


def test_served_requests_mix_and_arrivals():
    reqs = scenes.served_requests(600, 2000.0, 9, n_scenes=12, lo=1000, hi=20000, ray_lo=1000, ray_hi=20000)
    at = np.array([r[0] for r in reqs])
    assert np.all(np.diff(at) >= 0)  # arrival order
    kinds = [r[1] for r in reqs]
    assert kinds[:12] == ["build"] * 12 and [r[2] for r in reqs[:12]] == list(range(12))  # one build per scene first
    rest = kinds[12:]
    frac = {k: rest.count(k) / len(rest) for k in ("trace", "refit", "build")}
    assert abs(frac["trace"] - 0.7) < 0.06 and abs(frac["refit"] - 0.2) < 0.06 and abs(frac["build"] - 0.1) < 0.05
    for _, kind, scene, data in reqs:
        assert 0 <= scene < 12
        if kind == "trace":
            assert data.shape[1] == 8 and 1000 <= data.shape[0] <= 20000
        else:
            assert data.shape[1] == 12 and data.shape[0] == reqs[scene][3].shape[0]  # a scene keeps its count
    again = scenes.served_requests(600, 2000.0, 9, n_scenes=12, lo=1000, hi=20000, ray_lo=1000, ray_hi=20000)
    assert all(a[:3] == b[:3] and a[3].tobytes() == b[3].tobytes() for a, b in zip(reqs, again))
