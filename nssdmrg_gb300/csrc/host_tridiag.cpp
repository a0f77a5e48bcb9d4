// Lowest eigenpairs of a symmetric tridiagonal matrix (Lanczos T_m), host side.
//
// Eigenvalues by multisection on Sturm counts of the LDL^T pivots
//     q_0 = a_0 - x,   q_i = (a_i - x) - b_{i-1}^2 / q_{i-1},
// (the number of negative q_i is the number of eigenvalues below x; a pivot
// smaller than pivmin is replaced by -pivmin, the safeguard of LAPACK's
// bisection), four points per round evaluated as independent chains so the
// divisions overlap.  Eigenvectors by inverse iteration with the tridiagonal
// LU factorisation with partial pivoting (two solves from a fixed start
// vector), Gram-Schmidt against the vectors already found in the same
// cluster.
#include "host_tridiag.hpp"
#include <vector>
#include <limits>

#include <algorithm>
#include <cfloat>
#include <cmath>

namespace nss {

namespace {

constexpr double EPS = DBL_EPSILON;

// counts of eigenvalues below x[0..3]
inline void sturm4(const double *a, const double *b2, int m, const double *x, double pivmin, int *cnt) {
    double q0 = a[0] - x[0], q1 = a[0] - x[1], q2 = a[0] - x[2], q3 = a[0] - x[3];
    if (std::fabs(q0) < pivmin) q0 = -pivmin;
    if (std::fabs(q1) < pivmin) q1 = -pivmin;
    if (std::fabs(q2) < pivmin) q2 = -pivmin;
    if (std::fabs(q3) < pivmin) q3 = -pivmin;
    int c0 = q0 < 0.0, c1 = q1 < 0.0, c2 = q2 < 0.0, c3 = q3 < 0.0;
    for (int i = 1; i < m; ++i) {
        const double ai = a[i], bb = b2[i - 1];
        q0 = (ai - x[0]) - bb / q0;
        q1 = (ai - x[1]) - bb / q1;
        q2 = (ai - x[2]) - bb / q2;
        q3 = (ai - x[3]) - bb / q3;
        if (std::fabs(q0) < pivmin) q0 = -pivmin;
        if (std::fabs(q1) < pivmin) q1 = -pivmin;
        if (std::fabs(q2) < pivmin) q2 = -pivmin;
        if (std::fabs(q3) < pivmin) q3 = -pivmin;
        c0 += q0 < 0.0;
        c1 += q1 < 0.0;
        c2 += q2 < 0.0;
        c3 += q3 < 0.0;
    }
    cnt[0] = c0;
    cnt[1] = c1;
    cnt[2] = c2;
    cnt[3] = c3;
}

inline int sturm1(const double *a, const double *b2, int m, double x, double pivmin) {
    const double xs[4] = {x, x, x, x};
    int c[4];
    sturm4(a, b2, m, xs, pivmin, c);
    return c[0];
}

// eigenvalue e (0-based, ascending) inside [lo, hi] with count(lo) <= e < count(hi)
double multisect(const double *a, const double *b2, int m, int e, double lo, double hi, double pivmin) {
    for (int round = 0; round < 80; ++round) {
        const double w = hi - lo;
        if (!(w > 4.0 * EPS * std::max(std::fabs(lo), std::fabs(hi)) + 2.0 * pivmin)) break;
        double x[4];
        for (int k = 0; k < 4; ++k) x[k] = lo + w * (double)(k + 1) * 0.2;
        int c[4];
        sturm4(a, b2, m, x, pivmin, c);
        int k = 0;
        while (k < 4 && c[k] <= e) ++k;
        const double nlo = (k == 0) ? lo : x[k - 1];
        const double nhi = (k == 4) ? hi : x[k];
        if (nlo == lo && nhi == hi) break;   // no representable progress
        lo = nlo;
        hi = nhi;
    }
    return 0.5 * (lo + hi);
}

// y <- (T - sigma I)^{-1} y with the LU factors of T - sigma I (partial pivoting)
struct TriLU {
    std::vector<double> d, du, du2, dl;
    std::vector<char> piv;
    int m = 0;
    void factor(const double *a, const double *b, int m_, double sigma, double tiny) {
        m = m_;
        d.assign(m, 0.0);
        du.assign(m, 0.0);
        du2.assign(m, 0.0);
        dl.assign(m, 0.0);
        piv.assign(m, 0);
        for (int i = 0; i < m; ++i) d[i] = a[i] - sigma;
        for (int i = 0; i + 1 < m; ++i) {
            du[i] = b[i];
            dl[i] = b[i];
        }
        for (int i = 0; i + 1 < m; ++i) {
            if (std::fabs(d[i]) >= std::fabs(dl[i])) {
                if (d[i] == 0.0) d[i] = tiny;
                const double l = dl[i] / d[i];
                dl[i] = l;
                d[i + 1] -= l * du[i];
            } else {
                const double l = d[i] / dl[i];
                d[i] = dl[i];
                dl[i] = l;
                const double t = du[i];
                du[i] = d[i + 1];
                d[i + 1] = t - l * d[i + 1];
                if (i + 2 < m) {
                    du2[i] = du[i + 1];
                    du[i + 1] = -l * du[i + 1];
                }
                piv[i] = 1;
            }
        }
        if (d[m - 1] == 0.0) d[m - 1] = tiny;
    }
    void solve(double *y) const {
        for (int i = 0; i + 1 < m; ++i) {
            if (!piv[i]) {
                y[i + 1] -= dl[i] * y[i];
            } else {
                const double t = y[i];
                y[i] = y[i + 1];
                y[i + 1] = t - dl[i] * y[i + 1];
            }
        }
        y[m - 1] /= d[m - 1];
        if (m > 1) y[m - 2] = (y[m - 2] - du[m - 2] * y[m - 1]) / d[m - 2];
        for (int i = m - 3; i >= 0; --i) y[i] = (y[i] - du[i] * y[i + 1] - du2[i] * y[i + 2]) / d[i];
    }
};

void normalize(double *y, int m) {
    double big = 0.0;
    for (int i = 0; i < m; ++i) big = std::max(big, std::fabs(y[i]));
    if (!(big > 0.0) || !std::isfinite(big)) {
        for (int i = 0; i < m; ++i) y[i] = 1.0;
        big = 1.0;
    }
    double ss = 0.0;
    for (int i = 0; i < m; ++i) {
        y[i] /= big;
        ss += y[i] * y[i];
    }
    const double inv = 1.0 / std::sqrt(ss);
    for (int i = 0; i < m; ++i) y[i] *= inv;
}

}  // namespace

void tridiag_lowest(const double *a, const double *b, int m, int ne, double b_last, double *theta, double *s,
                    double *resid, const double *upper, std::vector<double> &work) {
    if (m <= 0 || ne <= 0) return;
    ne = std::min(ne, m);
    // work on 2^k T with ||2^k T|| ~ 1 (exact scaling), so that b^2 neither
    // underflows nor overflows
    double amax = 0.0;
    for (int i = 0; i < m; ++i) amax = std::max(amax, std::fabs(a[i]));
    for (int i = 0; i + 1 < m; ++i) amax = std::max(amax, std::fabs(b[i]));
    int ex = 0;
    if (amax > 0.0 && std::isfinite(amax)) std::frexp(amax, &ex);
    work.resize((size_t)3 * m);
    double *as = work.data(), *bs = as + m, *b2 = bs + m;
    for (int i = 0; i < m; ++i) as[i] = std::ldexp(a[i], -ex);
    for (int i = 0; i + 1 < m; ++i) bs[i] = std::ldexp(b[i], -ex);
    a = as;
    b = bs;
    double gl = a[0], gu = a[0], bmax2 = 0.0;
    for (int i = 0; i < m; ++i) {
        const double r = (i > 0 ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < m ? std::fabs(b[i]) : 0.0);
        gl = std::min(gl, a[i] - r);
        gu = std::max(gu, a[i] + r);
        if (i + 1 < m) {
            b2[i] = b[i] * b[i];
            bmax2 = std::max(bmax2, b2[i]);
        }
    }
    const double tnorm = std::max(std::fabs(gl), std::fabs(gu));
    const double pivmin = DBL_MIN * std::max(1.0, bmax2);
    const double pad = 2.0 * EPS * tnorm * (double)m + 2.0 * pivmin;
    gl -= pad;
    gu += pad;
    for (int e = 0; e < ne; ++e) {
        double lo = gl, hi = gu;
        if (e > 0) {
            const double c = theta[e - 1] - 4.0 * EPS * std::fabs(theta[e - 1]) - pivmin;
            if (c > lo && sturm1(a, b2, m, c, pivmin) <= e) lo = c;
        }
        if (upper) {
            // a Ritz value only moves down as m grows, and little once it has
            // settled: try narrow brackets below the previous value first
            const double ue = std::ldexp(upper[e], -ex);
            const double c = ue + 4.0 * EPS * std::fabs(ue) + pivmin;
            if (c < hi && c > lo && sturm1(a, b2, m, c, pivmin) > e) {
                hi = c;
                double d = std::max(1e-7 * std::fabs(c), 1e-12 * tnorm) + pivmin;
                for (int t = 0; t < 3; ++t, d *= 1e3) {
                    const double l2 = c - d;
                    if (l2 <= lo) break;
                    if (sturm1(a, b2, m, l2, pivmin) <= e) {
                        lo = l2;
                        break;
                    }
                }
            }
        }
        theta[e] = multisect(a, b2, m, e, lo, hi, pivmin);
    }
    TriLU lu;
    const double tiny = EPS * std::max(tnorm, DBL_MIN);
    const double clus = 1e-3 * std::max(tnorm, DBL_MIN);
    for (int e = 0; e < ne; ++e) {
        double *y = s + (size_t)e * m;
        for (int i = 0; i < m; ++i) y[i] = 1.0 + 0.01 * (double)((i * 7 + e * 3) % 11);
        lu.factor(a, b, m, theta[e], tiny);
        for (int it = 0; it < 2; ++it) {
            normalize(y, m);
            lu.solve(y);
            for (int f = 0; f < e; ++f) {
                if (std::fabs(theta[e] - theta[f]) > clus) continue;
                const double *z = s + (size_t)f * m;
                double dot = 0.0;
                for (int i = 0; i < m; ++i) dot += y[i] * z[i];
                for (int i = 0; i < m; ++i) y[i] -= dot * z[i];
            }
        }
        normalize(y, m);
        int imax = 0;
        for (int i = 1; i < m; ++i)
            if (std::fabs(y[i]) > std::fabs(y[imax])) imax = i;
        if (y[imax] < 0.0)
            for (int i = 0; i < m; ++i) y[i] = -y[i];
        resid[e] = std::fabs(b_last * y[m - 1]);
    }
    for (int e = 0; e < ne; ++e) theta[e] = std::ldexp(theta[e], ex);
}

}  // namespace nss

namespace nss {

namespace {

// y = (T - lam I)^{-1} m for T - lam I positive definite (LDL^T, no pivoting);
// returns false when a pivot is not positive (lam not below lambda_min(T))
bool spd_solve(const double *a, const double *b, int k, double lam, const double *m, double *y, double *d) {
    for (int i = 0; i < k; ++i) {
        double di = a[i] - lam;
        if (i > 0) di -= b[i - 1] * b[i - 1] / d[i - 1];
        if (!(di > 0.0)) return false;
        d[i] = di;
    }
    // forward: z_i = m_i - (b_{i-1}/d_{i-1}) z_{i-1}
    for (int i = 0; i < k; ++i) y[i] = m[i] - (i > 0 ? b[i - 1] / d[i - 1] * y[i - 1] : 0.0);
    // diagonal and backward: y_i = z_i/d_i - (b_i/d_i) y_{i+1}
    for (int i = k - 1; i >= 0; --i) y[i] = y[i] / d[i] - (i + 1 < k ? b[i] / d[i] * y[i + 1] : 0.0);
    return true;
}

}  // namespace

bool arrow_lowest(double theta0, const double *m, const double *a, const double *b, int k, double b_last,
                  double *lam, double *c, double *resid, std::vector<double> &work) {
    c[0] = 1.0;
    if (k <= 0) {
        *lam = theta0;
        *resid = 0.0;
        return true;
    }
    work.resize((size_t)4 * k + 16);
    double *y = work.data(), *d = y + k, *tw = d + k;
    // upper end of the bracket: min(theta0, lambda_min(T)), the latter by
    // the tridiagonal solver (its eigenvector scratch in tw)
    double tmin = 0.0, tres = 0.0;
    std::vector<double> w2;
    std::vector<double> s1((size_t)k);
    tridiag_lowest(a, b, k, 1, 0.0, &tmin, s1.data(), &tres, nullptr, w2);
    double hi = std::min(theta0, tmin);
    // lower end: Gershgorin bound of M
    double msum = 0.0;
    for (int i = 0; i < k; ++i) msum += std::fabs(m[i]);
    double lo = theta0 - msum;
    for (int i = 0; i < k; ++i) {
        const double r = (i > 0 ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < k ? std::fabs(b[i]) : 0.0) + std::fabs(m[i]);
        lo = std::min(lo, a[i] - r);
    }
    const double scale = std::max({std::fabs(lo), std::fabs(hi), DBL_MIN});
    lo -= 4.0 * EPS * scale;
    // step just below hi so that T - lam I stays definite
    double x = hi - std::max(1e-12 * scale, 4.0 * EPS * scale);
    if (x <= lo) x = 0.5 * (lo + hi);
    (void)tw;
    bool ok = false;
    for (int it = 0; it < 200; ++it) {
        if (!spd_solve(a, b, k, x, m, y, d)) {   // above lambda_min(T): move down
            hi = x;
            x = 0.5 * (lo + hi);
            continue;
        }
        double my = 0.0, yy = 0.0;
        for (int i = 0; i < k; ++i) {
            my += m[i] * y[i];
            yy += y[i] * y[i];
        }
        const double f = theta0 - x - my;
        if (f > 0.0) lo = x;
        else hi = x;
        const double step = f / (1.0 + yy);      // Newton: f' = -(1 + y.y)
        double xn = x + step;
        if (!(xn > lo && xn < hi)) xn = 0.5 * (lo + hi);
        const double dx = std::fabs(xn - x);
        x = xn;
        if (dx <= 2.0 * EPS * std::fabs(x) || hi - lo <= 4.0 * EPS * std::fabs(x)) {
            ok = spd_solve(a, b, k, x, m, y, d);
            break;
        }
    }
    if (!ok) return false;
    double nn = 1.0;
    for (int i = 0; i < k; ++i) nn += y[i] * y[i];
    const double inv = 1.0 / std::sqrt(nn);
    c[0] = inv;
    for (int i = 0; i < k; ++i) c[i + 1] = -y[i] * inv;
    *lam = x;
    *resid = std::fabs(b_last * c[k]);
    return true;
}

// Implicit QL with Wilkinson shifts for a symmetric tridiagonal matrix
// (Bowdler, Martin, Reinsch and Wilkinson, "The QR and QL algorithms for
// symmetric matrices", Numer. Math. 11 (1968)).  Work is O(n^2) for the
// eigenvalues and O(n^3) for the accumulated rotations; each rotation
// touches two contiguous columns of Z.
bool tridiag_ql(int n, double *d, double *e, double *Z) {
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) Z[(size_t)j * n + i] = i == j ? 1.0 : 0.0;
    if (n <= 1) return true;
    std::vector<double> off(n, 0.0);
    for (int i = 0; i + 1 < n; ++i) off[i] = e[i];
    const double eps = std::numeric_limits<double>::epsilon();
    for (int l = 0; l < n; ++l) {
        for (int iter = 0;; ++iter) {
            int m = l;
            for (; m + 1 < n; ++m) {                 // a negligible coupling splits the matrix at m
                const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
                if (std::fabs(off[m]) <= eps * dd) break;
            }
            if (m == l) break;
            if (iter == 60) return false;
            // shift: the eigenvalue of the leading 2x2 block nearer d[l]
            double g = (d[l + 1] - d[l]) / (2.0 * off[l]);
            double r = std::hypot(g, 1.0);
            g = d[m] - d[l] + off[l] / (g + std::copysign(r, g));
            double s = 1.0, c = 1.0, p = 0.0;
            int i = m - 1;
            bool split = false;
            for (; i >= l; --i) {                    // chase the bulge from m up to l
                const double f = s * off[i], b = c * off[i];
                r = std::hypot(f, g);
                off[i + 1] = r;
                if (r == 0.0) {                      // exact underflow: deflate and restart
                    d[i + 1] -= p;
                    off[m] = 0.0;
                    split = true;
                    break;
                }
                s = f / r;
                c = g / r;
                g = d[i + 1] - p;
                r = (d[i] - g) * s + 2.0 * c * b;
                p = s * r;
                d[i + 1] = g + p;
                g = c * r - b;
                double *zi = Z + (size_t)i * n, *zj = Z + (size_t)(i + 1) * n;
                for (int k = 0; k < n; ++k) {
                    const double t = zj[k];
                    zj[k] = s * zi[k] + c * t;
                    zi[k] = c * zi[k] - s * t;
                }
            }
            if (split) continue;
            d[l] -= p;
            off[l] = g;
            off[m] = 0.0;
        }
    }
    // ascending order, vectors along
    std::vector<int> ord(n);
    for (int j = 0; j < n; ++j) ord[j] = j;
    std::sort(ord.begin(), ord.end(), [&](int x, int y) { return d[x] < d[y]; });
    std::vector<double> ds(n), Zs((size_t)n * n);
    for (int j = 0; j < n; ++j) {
        ds[j] = d[ord[j]];
        std::copy(Z + (size_t)ord[j] * n, Z + (size_t)(ord[j] + 1) * n, Zs.begin() + (size_t)j * n);
    }
    std::copy(ds.begin(), ds.end(), d);
    std::copy(Zs.begin(), Zs.end(), Z);
    return true;
}

}  // namespace nss
