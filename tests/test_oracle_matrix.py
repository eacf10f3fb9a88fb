"""CPU checks of the oracle's Horn and Long restatements (matrix/{horn,long}.rs, float64).

The oracle follows the reference's steps literally; the GPU library reaches the same
quantities through exact identities (its m x m forms).  These tests pin the oracle's literal
steps against those identities, so that a GPU result that matches the oracle is also the
identity-based algorithm's result:
  - G_pinv = V diag(s / (s^2 + a^2)) U^H equals G^H (G G^H + a^2 I)^-1;
  - MM = P (I - G G_pinv) P equals a^2 P (G G^H + a^2 I)^-1 P;
  - Long's QR solve of the normal equations equals the Woodbury form
    S^-1 G^H (I + G S^-1 G^H)^-1 f;
and check the SDP's invariants and the coordinate order."""
import numpy as np
import pytest

import oracle as O
import workloads as W


def _g(m, seed):
    rng = np.random.default_rng(seed)
    w, foci, amps = W.gspat_request(rng, m)
    s = w.sources.copy()
    s[:, 7] = 0.0
    return O.build_g_f64(1, s, w.k, w.atten, foci), amps.astype(np.float64), w, foci


@pytest.mark.parametrize("m", [2, 8, 31])
def test_horn_pinv_and_mm_identities(m):
    g, amps, _, _ = _g(m, 500 + m)
    a2 = 1e-10
    mm, g_pinv = O.horn_mm_f64(g, amps)
    kinv = np.linalg.inv(g @ g.conj().T + a2 * np.eye(m))
    pinv2 = g.conj().T @ kinv
    assert np.max(np.abs(g_pinv - pinv2)) <= 1e-9 * np.max(np.abs(pinv2))
    mm2 = a2 * np.diag(amps) @ kinv @ np.diag(amps)
    # the literal form loses digits to the subtraction I - G G_pinv (entries ~1e-9 of 1)
    err = np.max(np.abs(mm - mm2)) / np.max(np.abs(mm2))
    print(f"m={m}: MM literal vs identity {err:.2e}")
    assert err <= 1e-4


def test_horn_sdp_keeps_x_hermitian_with_unit_diagonal():
    g, amps, _, _ = _g(8, 511)
    mm, _ = O.horn_mm_f64(g, amps)
    x = O.horn_sdp_f64(mm, O.horn_indices(8, 800))
    np.testing.assert_allclose(x, x.conj().T, atol=0)
    np.testing.assert_array_equal(np.diag(x), np.ones(8))
    # the SDP is invariant to the scale of MM
    x2 = O.horn_sdp_f64(mm * 1e7, O.horn_indices(8, 800))
    assert np.max(np.abs(x - x2)) <= 1e-9 * np.max(np.abs(x))


def test_horn_indices_cover_the_foci_deterministically():
    idx = O.horn_indices(64, 6400)
    assert idx.min() == 0 and idx.max() == 63
    np.testing.assert_array_equal(idx, O.horn_indices(64, 6400))
    counts = np.bincount(idx, minlength=64)
    assert counts.min() > 50 and counts.max() < 160  # about 100 each


@pytest.mark.parametrize("m", [2, 8, 31])
def test_long_qr_solve_equals_woodbury(m):
    g, amps, w, foci = _g(m, 520 + m)
    n = g.shape[1]
    _, q = O.long_f64(1, w.sources, w.k, w.atten, foci, amps)
    sig2 = (np.abs(g) * amps[:, None]).sum(axis=0) / m
    # f from the same e_arg: recover it from the literal solution's residual-free target
    denomi = g.sum(axis=1)
    r = g @ (amps[:, None] * g.conj() / denomi[:, None]).T
    wv, v = np.linalg.eigh(r, UPLO="L")
    e_arg = np.angle(O._phase_fixed(v)[int(np.argmax(wv)), :])
    f = amps * np.exp(1j * e_arg)
    y = np.linalg.solve(np.eye(m) + (g / sig2) @ g.conj().T, f)
    q2 = (g.conj().T @ y) / sig2
    err = np.max(np.abs(q - q2)) / np.max(np.abs(q2))
    print(f"m={m}, n={n}: QR vs Woodbury {err:.2e}")
    assert err <= 1e-8


def test_phase_rule_makes_eigenvectors_unique():
    rng = np.random.default_rng(3)
    a = rng.normal(size=(6, 6)) + 1j * rng.normal(size=(6, 6))
    h = a + a.conj().T
    _, v = np.linalg.eigh(h)
    ph = np.exp(1j * rng.uniform(-np.pi, np.pi, 6))
    np.testing.assert_allclose(O._phase_fixed(v), O._phase_fixed(v * ph), atol=1e-12)
    first = O._phase_fixed(v)[0]
    assert np.all(first.real > 0) and np.all(first.imag == 0)
