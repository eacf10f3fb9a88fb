// Small dense complex linear algebra on the host, in double: the k x k systems of the
// optimizers whose O(n m) and O(n m^2) work runs on the device (apo.cu, matrix.cu).  Matrices
// are row-major std::vector<std::complex<double>>.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

namespace afc {
namespace dense {

using cd = std::complex<double>;

// Cholesky factorisation in place of the Hermitian positive definite k x k matrix a: its lower
// triangle becomes L with a = L L^H (the diagonal real).  False if a is not positive definite.
inline bool hpd_factor(std::vector<cd>& a, int k) {
    for (int j = 0; j < k; ++j) {
        double d = a[j * k + j].real();
        for (int p = 0; p < j; ++p) d -= std::norm(a[j * k + p]);
        if (!(d > 0.0)) return false;
        d = std::sqrt(d);
        a[j * k + j] = d;
        for (int i = j + 1; i < k; ++i) {
            cd s = a[i * k + j];
            for (int p = 0; p < j; ++p) s -= a[i * k + p] * std::conj(a[j * k + p]);
            a[i * k + j] = s / d;
        }
    }
    return true;
}

// Solve L L^H c = b in place for one right-hand side, L from hpd_factor.
inline void hpd_substitute(const std::vector<cd>& l, std::vector<cd>& b, int k) {
    for (int i = 0; i < k; ++i) {
        cd s = b[i];
        for (int p = 0; p < i; ++p) s -= l[i * k + p] * b[p];
        b[i] = s / l[i * k + i].real();
    }
    for (int i = k - 1; i >= 0; --i) {
        cd s = b[i];
        for (int p = i + 1; p < k; ++p) s -= std::conj(l[p * k + i]) * b[p];
        b[i] = s / l[i * k + i].real();
    }
}

// Solve the Hermitian positive definite system a c = b (k x k, a overwritten by its factor).
inline bool hpd_solve(std::vector<cd>& a, std::vector<cd>& b, int k) {
    if (!hpd_factor(a, k)) return false;
    hpd_substitute(a, b, k);
    return true;
}

// Inverse of the Hermitian positive definite k x k matrix a (overwritten by its factor) into
// inv, column by column.
inline bool hpd_inverse(std::vector<cd>& a, std::vector<cd>& inv, int k) {
    if (!hpd_factor(a, k)) return false;
    inv.assign(static_cast<size_t>(k) * k, cd(0.0, 0.0));
    std::vector<cd> col(k);
    for (int c = 0; c < k; ++c) {
        for (int i = 0; i < k; ++i) col[i] = cd(i == c ? 1.0 : 0.0, 0.0);
        hpd_substitute(a, col, k);
        for (int i = 0; i < k; ++i) inv[i * k + c] = col[i];
    }
    return true;
}

// Cyclic Jacobi eigendecomposition of the Hermitian k x k matrix a (row-major, destroyed; only
// its lower triangle and the real part of its diagonal are read, the upper triangle is taken as
// the conjugate of the lower).  Eigenvalues go to lam, unit eigenvectors to the columns of v.
//
// Pivot (p, q) with a_qp = |b| e^{-i phi} (so a_pq = |b| e^{i phi}) is annihilated by the
// unitary J with J_pp = J_qq = c, J_pq = s e^{i phi}, J_qp = -s e^{-i phi}, where t = s / c is
// the smaller root of t^2 + 2 theta t - 1 = 0, theta = (a_qq - a_pp) / (2 |b|): the real
// symmetric rotation after a diagonal phase change.
//
// The eigenpairs are then put in ascending order of eigenvalue (ties keep their order), and
// each eigenvector's phase is fixed: its first nonzero entry is real and positive.  Eigenvectors
// are defined only up to such a unit factor, and an order is a choice too, so both rules are
// part of what a caller gets.
inline void hermitian_eigen(std::vector<cd>& a, int k, std::vector<double>& lam,
                            std::vector<cd>& v) {
    for (int i = 0; i < k; ++i) {
        a[i * k + i] = cd(a[i * k + i].real(), 0.0);
        for (int j = i + 1; j < k; ++j) a[i * k + j] = std::conj(a[j * k + i]);
    }
    v.assign(static_cast<size_t>(k) * k, cd(0.0, 0.0));
    for (int i = 0; i < k; ++i) v[i * k + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) {
                const double x = std::norm(a[i * k + j]);
                tot += x;
                if (i != j) off += x;
            }
        if (off == 0.0 || off <= 1e-30 * tot) break;
        for (int p = 0; p < k; ++p)
            for (int q = p + 1; q < k; ++q) {
                const cd apq = a[p * k + q];
                const double b = std::abs(apq);
                if (b == 0.0) continue;
                const cd e = apq / b;  // e^{i phi}
                const double theta = (a[q * k + q].real() - a[p * k + p].real()) / (2.0 * b);
                const double t = (theta >= 0 ? 1.0 : -1.0) /
                                 (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                const cd se = s * e, sec = s * std::conj(e);
                for (int r = 0; r < k; ++r) {  // a J: columns p, q
                    const cd arp = a[r * k + p], arq = a[r * k + q];
                    a[r * k + p] = c * arp - sec * arq;
                    a[r * k + q] = se * arp + c * arq;
                }
                for (int r = 0; r < k; ++r) {  // J^H (a J): rows p, q
                    const cd apr = a[p * k + r], aqr = a[q * k + r];
                    a[p * k + r] = c * apr - se * aqr;
                    a[q * k + r] = sec * apr + c * aqr;
                }
                a[p * k + q] = a[q * k + p] = 0.0;
                a[p * k + p] = cd(a[p * k + p].real(), 0.0);
                a[q * k + q] = cd(a[q * k + q].real(), 0.0);
                for (int r = 0; r < k; ++r) {  // v J
                    const cd vrp = v[r * k + p], vrq = v[r * k + q];
                    v[r * k + p] = c * vrp - sec * vrq;
                    v[r * k + q] = se * vrp + c * vrq;
                }
            }
    }
    std::vector<int> order(k);
    for (int i = 0; i < k; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return a[x * k + x].real() < a[y * k + y].real();
    });
    lam.resize(k);
    std::vector<cd> vs(static_cast<size_t>(k) * k);
    for (int j = 0; j < k; ++j) {
        const int o = order[j];
        lam[j] = a[o * k + o].real();
        for (int r = 0; r < k; ++r) vs[r * k + j] = v[r * k + o];
    }
    v.swap(vs);
    for (int j = 0; j < k; ++j) {  // phase rule: the first nonzero entry real and positive
        int r0 = 0;
        while (r0 < k && v[r0 * k + j] == cd(0.0, 0.0)) ++r0;
        if (r0 == k) continue;
        const double mag = std::abs(v[r0 * k + j]);
        const cd ph = std::conj(v[r0 * k + j]) / mag;
        for (int r = 0; r < k; ++r) v[r * k + j] *= ph;
        v[r0 * k + j] = mag;
    }
}

}  // namespace dense
}  // namespace afc
