"""Seeded workload generators (CPU): assembly placements and request streams."""
import math

import numpy as np

from dpx import workloads as W


def _euler(a, b, c):
    c1, s1, c2, s2, c3, s3 = math.cos(a), math.sin(a), math.cos(b), math.sin(b), math.cos(c), math.sin(c)
    return np.array([[c2 * c3, -c2 * s3, s2], [c1 * s3 + c3 * s1 * s2, c1 * c3 - s1 * s2 * s3, -c2 * s1],
                     [s1 * s3 - c1 * c3 * s2, c3 * s1 + c1 * s2 * s3, c1 * c2]])


def test_icosahedral_group():
    g = W.icosahedral_rotations()
    assert len(g) == 60
    for R in g:
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-12) and abs(np.linalg.det(R) - 1) < 1e-12
        assert np.allclose(_euler(*W.euler_from_matrix(R)), R, atol=1e-12)
    # closed under products
    for A in g[::7]:
        for B in g[::5]:
            assert any(np.allclose(A @ B, C, atol=1e-9) for C in g)
    rot, tr = W.icosahedral_copies(12.0)
    assert rot.shape == (60, 3) and np.allclose(np.linalg.norm(tr, axis=1), 12.0)


def test_helix_copies_screw_symmetry():
    rot, tr = W.helix_copies(1000, 12.0, 13, 8.0, seed=3)
    assert len({tuple(r) for r in rot}) == 13  # exact repeats: 13 rotation groups
    assert np.allclose(np.hypot(tr[:, 0], tr[:, 1]), 12.0)
    assert abs(tr[13, 2] - 8.0) < 1e-12
    # copy k's rotation is Rz(azimuth) R0
    R0 = _euler(*rot[0])
    for k in (1, 5, 12):
        a = 2 * math.pi * k / 13
        Rz = np.array([[math.cos(a), -math.sin(a), 0], [math.sin(a), math.cos(a), 0], [0, 0, 1]])
        assert np.allclose(_euler(*rot[k]), Rz @ R0, atol=1e-12)
    rr, _ = W.helix_copies(50, screw=False, seed=4)
    assert len({tuple(r) for r in rr}) == 50


def test_batch_mix_statistics():
    mix = W.batch_mix(512)
    a = np.array([s.atoms for s in mix])
    assert a.min() >= 500 and a.max() <= 200_000
    assert sum(s.solvent for s in mix) == 256
    assert all(40 <= s.layers <= 250 and 2 <= s.qmax <= 10 for s in mix)
    assert [s.atoms for s in W.batch_mix(512)] == list(a)  # seeded


def test_request_stream_shape():
    s = W.request_stream(60, rate_hz=200.0, helix_copies_n=2000)
    kinds = [r.kind for r in s]
    assert set(kinds) <= {"subunit", "assembly", "helix"}
    assert all(b.arrival_s > a.arrival_s for a, b in zip(s, s[1:]))
    for j, r in enumerate(s):
        if r.repeat_of >= 0:
            base = s[r.repeat_of]
            assert base.leaf is r.leaf and base.grid_size == r.grid_size and r.repeat_of < j
        assert r.Q[-1] <= r.qmax + 1e-12
    assert 0 < sum(r.repeat_of >= 0 for r in s) < len(s)


def test_oracle_globule_is_the_library_globule():
    """The CPU baseline builds its structure with the oracle's generator (no
    library loaded); it must be the library's globule bit for bit."""
    import oracle as O
    from dpx import models as M
    from dpx.elements import GLOBULE_CODES
    for n, r, seed in ((2000, 2.5, 20250), (5000, 3.0, 2020), (700, 1.4, 9)):
        el, xyz = O.make_globule(n, r, seed)
        sym, xyz_lib = M.make_globule(n, r, seed)
        assert np.array_equal(xyz.astype(np.float64), xyz_lib)
        assert [GLOBULE_CODES[e] for e in el] == sym
