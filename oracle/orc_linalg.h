// Oracle (test infrastructure only): the small dense solvers that stand in for
// Eigen's in the CPU restatement (orc_icp.cpp) and in the Eigen-API shim
// (eigen_shim/) that the reference's own sources compile against here.
// Written from the mathematics; one implementation serves both, so the two
// CPU builds solve identically.
//
//   jacobi_eigen   symmetric eigenvalues (ascending) and eigenvectors, cyclic
//                  Jacobi in double (stands in for SelfAdjointEigenSolver)
//   ldlt_solve6    6x6 LDL^T with symmetric diagonal pivoting, float (ldlt())
//   svd3           3x3 SVD from the eigenvectors of M^T M, singular values
//                  descending (JacobiSVD's order)
//   inverse4_rm    4x4 inverse by the adjugate of 2x2 minors, float, row-major
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>

#include "orc_math.h"

namespace orc {
namespace linalg {

inline void jacobi_eigen(int n, double* a /* n*n row-major, destroyed */, double* ev, double* vec /* n*n or null */) {
    if (vec)
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) vec[i * n + j] = (i == j);
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = i + 1; j < n; ++j) off += a[i * n + j] * a[i * n + j];
        if (off < 1e-300) break;
        for (int p = 0; p < n; ++p) {
            for (int q = p + 1; q < n; ++q) {
                const double apq = a[p * n + q];
                if (apq == 0.0) continue;
                const double theta = (a[q * n + q] - a[p * n + p]) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {
                    const double akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = c * akp - s * akq;
                    a[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = c * apk - s * aqk;
                    a[q * n + k] = s * apk + c * aqk;
                }
                if (vec)
                    for (int k = 0; k < n; ++k) {
                        const double vkp = vec[k * n + p], vkq = vec[k * n + q];
                        vec[k * n + p] = c * vkp - s * vkq;
                        vec[k * n + q] = s * vkp + c * vkq;
                    }
            }
        }
    }
    for (int i = 0; i < n; ++i) ev[i] = a[i * n + i];
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j)
            if (ev[j] < ev[i]) {
                std::swap(ev[i], ev[j]);
                if (vec)
                    for (int k = 0; k < n; ++k) std::swap(vec[k * n + i], vec[k * n + j]);
            }
}

inline void ldlt_solve6(const float A_in[36], const float b[6], float x[6]) {
    float A[36];
    std::memcpy(A, A_in, sizeof(A));
    int perm[6] = {0, 1, 2, 3, 4, 5};
    float L[36] = {0}, D[6];
    for (int k = 0; k < 6; ++k) {
        int p = k;
        for (int i = k + 1; i < 6; ++i)
            if (std::fabs(A[i * 6 + i]) > std::fabs(A[p * 6 + p])) p = i;
        if (p != k) {
            for (int j = 0; j < 6; ++j) std::swap(A[k * 6 + j], A[p * 6 + j]);
            for (int i = 0; i < 6; ++i) std::swap(A[i * 6 + k], A[i * 6 + p]);
            for (int j = 0; j < k; ++j) std::swap(L[k * 6 + j], L[p * 6 + j]);
            std::swap(perm[k], perm[p]);
        }
        D[k] = A[k * 6 + k];
        L[k * 6 + k] = 1.0f;
        for (int i = k + 1; i < 6; ++i) L[i * 6 + k] = A[i * 6 + k] / D[k];
        for (int i = k + 1; i < 6; ++i)
            for (int j = k + 1; j <= i; ++j) {
                A[i * 6 + j] -= L[i * 6 + k] * A[j * 6 + k];
                A[j * 6 + i] = A[i * 6 + j];
            }
        for (int i = k + 1; i < 6; ++i) A[i * 6 + k] = A[k * 6 + i] = 0.0f;
    }
    float y[6];
    for (int i = 0; i < 6; ++i) {
        float s = b[perm[i]];
        for (int j = 0; j < i; ++j) s -= L[i * 6 + j] * y[j];
        y[i] = s;
    }
    for (int i = 0; i < 6; ++i) y[i] /= D[i];
    float z[6];
    for (int i = 5; i >= 0; --i) {
        float s = y[i];
        for (int j = i + 1; j < 6; ++j) s -= L[j * 6 + i] * z[j];
        z[i] = s;
    }
    for (int i = 0; i < 6; ++i) x[perm[i]] = z[i];
}

// M = U diag(S) V^T (row-major 3x3, double), S descending.
inline void svd3(const double m[9], double U[9], double S[3], double V[9]) {
    double mtm[9], ev[3], Va[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += m[k * 3 + i] * m[k * 3 + j];
            mtm[i * 3 + j] = s;
        }
    jacobi_eigen(3, mtm, ev, Va);  // ascending
    for (int c = 0; c < 3; ++c) {
        const int src = 2 - c;  // descending
        S[c] = std::sqrt(std::max(ev[src], 1e-300));
        for (int i = 0; i < 3; ++i) V[i * 3 + c] = Va[i * 3 + src];
        for (int i = 0; i < 3; ++i) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += m[i * 3 + k] * V[k * 3 + c];
            U[i * 3 + c] = s / S[c];
        }
    }
}

inline void inverse4_rm(const float in[16], float out[16]) { inverse4(M4::from(in)).to(out); }

}  // namespace linalg
}  // namespace orc
