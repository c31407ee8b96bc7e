// Eigen-decomposition of the 1-D coarsest-level operators for the exact
// coarsest solve of the MIXED form (fast diagonalisation).
//
// The stretched 7-point operator of a level is a Kronecker sum of one 1-D
// operator per axis, A = Ax (+) Ay (+) Az, each tridiagonal (with corners
// on a periodic axis) once the ghost rule is folded in.  A 1-D operator
// whose off-diagonal pairs have positive products is similar to a
// symmetric matrix through a diagonal scaling D: S = D A D^-1.  With
// S = Q L Q^T (cyclic Jacobi rotations) the operator is A = V L V^-1 with
// V = D^-1 Q and V^-1 = Q^T D.
#include "grid_host.h"

#include <cmath>
#include <vector>

namespace saras {

namespace {

// Cyclic Jacobi eigenvalue iteration of a symmetric n x n matrix (row
// major, destroyed): eigenvalues in lam, eigenvectors in the columns of q.
void jacobi_eigen(int n, std::vector<double> &a, std::vector<double> &q, double *lam) {
    q.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; i++) q[(size_t)i * n + i] = 1.0;
    auto A = [&](int i, int j) -> double & { return a[(size_t)i * n + j]; };
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                tot += A(i, j) * A(i, j);
                if (i != j) off += A(i, j) * A(i, j);
            }
        if (off <= 1e-32 * tot) break;
        for (int p = 0; p < n; p++)
            for (int r = p + 1; r < n; r++) {
                const double apr = A(p, r);
                if (apr == 0.0) continue;
                const double theta = (A(r, r) - A(p, p)) / (2.0 * apr);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {  // A <- A J
                    const double akp = A(k, p), akr = A(k, r);
                    A(k, p) = c * akp - s * akr;
                    A(k, r) = s * akp + c * akr;
                }
                for (int k = 0; k < n; k++) {  // A <- J^T A
                    const double apk = A(p, k), ark = A(r, k);
                    A(p, k) = c * apk - s * ark;
                    A(r, k) = s * apk + c * ark;
                }
                for (int k = 0; k < n; k++) {
                    const double qkp = q[(size_t)k * n + p], qkr = q[(size_t)k * n + r];
                    q[(size_t)k * n + p] = c * qkp - s * qkr;
                    q[(size_t)k * n + r] = s * qkp + c * qkr;
                }
            }
    }
    for (int i = 0; i < n; i++) lam[i] = A(i, i);
}

}  // namespace

bool coarse_axis_eigen(int n, const double *cm, const double *cp, const double *a2, bool per, int sg_lo, int sg_hi,
                       double *V, double *Vi, double *lam) {
    // the 1-D operator: cm u(i-1) + cp u(i+1) - 2 a2 u(i), ghosts folded
    std::vector<double> A((size_t)n * n, 0.0);
    auto at = [&](int i, int j) -> double & { return A[(size_t)i * n + j]; };
    for (int i = 0; i < n; i++) {
        at(i, i) += -2.0 * a2[i];
        if (i > 0)
            at(i, i - 1) += cm[i];
        else if (per)
            at(0, n - 1) += cm[0];
        else
            at(0, 0) += sg_lo * cm[0];
        if (i < n - 1)
            at(i, i + 1) += cp[i];
        else if (per)
            at(n - 1, 0) += cp[n - 1];
        else
            at(n - 1, n - 1) += sg_hi * cp[n - 1];
    }
    // diagonal similarity along the chain: (d_{i+1}/d_i)^2 = A(i,i+1)/A(i+1,i)
    std::vector<double> d((size_t)n, 1.0);
    for (int i = 0; i + 1 < n; i++) {
        const double up = at(i, i + 1), lo = at(i + 1, i);
        if (!(up * lo > 0.0)) return false;
        d[(size_t)i + 1] = d[(size_t)i] * std::sqrt(up / lo);
    }
    std::vector<double> S((size_t)n * n);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) S[(size_t)i * n + j] = d[(size_t)i] * at(i, j) / d[(size_t)j];
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++) {
            const double x = S[(size_t)i * n + j], y = S[(size_t)j * n + i];
            if (std::fabs(x - y) > 1e-12 * (std::fabs(x) + std::fabs(y))) return false;  // e.g. stretched periodic
            S[(size_t)i * n + j] = S[(size_t)j * n + i] = 0.5 * (x + y);
        }
    std::vector<double> Q;
    jacobi_eigen(n, S, Q, lam);
    for (int i = 0; i < n; i++)
        for (int k = 0; k < n; k++) {
            V[(size_t)i * n + k] = Q[(size_t)i * n + k] / d[(size_t)i];
            Vi[(size_t)k * n + i] = Q[(size_t)i * n + k] * d[(size_t)i];
        }
    return true;
}

}  // namespace saras
