"""The oracle's APO (float64, C) against a second restatement of nls/apo.rs:36-158 in numpy with
the reference's explicit matrices, on 12-transducer problems that take 1 to 63 quasi-Newton
steps.  Both run the same float64 iteration, so they agree to the float32 rounding of the
output records."""
import numpy as np
import pytest

import oracle as O
import workloads as W


def _apo_numpy(G, amps, lam):
    m, n = G.shape
    p = amps.astype(np.complex128)
    p2 = np.abs(p) ** 2
    q = np.linalg.solve(G.conj().T @ G + lam * np.eye(n), G.conj().T @ p)
    R = [np.outer(G[i].conj(), G[i]) for i in range(m)]

    def J(v):
        return sum(abs(v.conj() @ R[i] @ v - p2[i]) ** 2 for i in range(m)) + abs(v @ v) * lam

    def grad(v):
        return sum((R[i] @ v) * (p2[i] - abs(v.conj() @ R[i] @ v)) for i in range(m)) + lam * v

    H = np.eye(n, dtype=np.complex128)
    g = grad(q)
    steps = 0
    for _ in range(200):
        d = -(H @ g)
        best, alpha = np.inf, 0.0
        for i in range(100):
            a = float(np.float32(i) / np.float32(100))
            v = J(q + a * d)
            if v < best:
                best, alpha = v, a
        d = d * alpha
        if np.linalg.norm(d) < 1e-8:
            break
        steps += 1
        qn = q + d
        gn = grad(qn)
        s = gn - g
        u = H @ s
        H = H + np.outer(d, d) / (d @ s) - np.outer(u, u) / (s @ u)
        q, g = qn, gn
    return q, steps


@pytest.mark.parametrize("seed", [0, 3, 4, 9])
def test_oracle_apo_matches_numpy_restatement(seed):
    rng = np.random.default_rng(seed)
    n, m = 12, 2
    pos = W.tiled_array(1, 1)[:n]
    rec = W.t4010a1_records(pos, 1.0, 0.0)
    k = np.full(n, W.wavenumber(), np.float32)
    a = np.zeros(n, np.float32)
    foci = np.array([[pos[:, 0].mean() + rng.uniform(-10, 10), pos[:, 1].mean(),
                      rng.uniform(30, 80)] for _ in range(m)], np.float32)
    amps = rng.uniform(0.01, 0.2, m).astype(np.float32)
    lam = float(10 ** rng.uniform(-6, -1))
    q, steps = _apo_numpy(O.build_g_f64(1, rec, k, a, foci), amps, lam)
    assert steps >= 1
    ref = O.apo_f64(1, rec, k, a, foci, amps, lam).reshape(-1, 9)
    camax = np.max(np.abs(q.real) + np.abs(q.imag))
    np.testing.assert_allclose(ref[:, 6], np.abs(q) / camax, rtol=0, atol=1e-6)
    dphi = np.angle(np.exp(1j * (np.angle(q) - ref[:, 7])))
    assert np.max(np.abs(dphi)) < 1e-5
