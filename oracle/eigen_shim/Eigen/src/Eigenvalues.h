// Oracle (test infrastructure only): SelfAdjointEigenSolver and JacobiSVD of
// the Eigen-API shim, on the restatement's solvers (oracle/orc_linalg.h).
#pragma once

namespace Eigen {

// Eigenvalues ascending, eigenvectors as columns (cyclic Jacobi in double).
template <typename MatrixType>
class SelfAdjointEigenSolver {
    static constexpr int N = MatrixType::RowsAtCompileTime;
    using T = typename MatrixType::Scalar;

public:
    explicit SelfAdjointEigenSolver(const MatrixType& A) {
        double a[N * N], ev[N], vec[N * N];
        bool finite = true;
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                a[i * N + j] = static_cast<double>(A(i, j));
                finite = finite && std::isfinite(a[i * N + j]);
            }
        info_ = finite ? Success : NoConvergence;
        orc::linalg::jacobi_eigen(N, a, ev, vec);
        for (int i = 0; i < N; ++i) {
            values_(i) = static_cast<T>(ev[i]);
            for (int j = 0; j < N; ++j) vectors_(i, j) = static_cast<T>(vec[i * N + j]);
        }
    }
    ComputationInfo info() const { return info_; }
    const Matrix<T, N, 1>& eigenvalues() const { return values_; }
    const MatrixType& eigenvectors() const { return vectors_; }

private:
    ComputationInfo info_;
    Matrix<T, N, 1> values_;
    MatrixType vectors_;
};

// Full SVD of a 3x3 matrix from the eigenvectors of M^T M (the restatement's
// method); U and V orthonormal, M = U S V^T.
template <typename MatrixType>
class JacobiSVD {
    using T = typename MatrixType::Scalar;

public:
    JacobiSVD(const MatrixType& M, unsigned int /*options*/) {
        static_assert(MatrixType::RowsAtCompileTime == 3 && MatrixType::ColsAtCompileTime == 3, "3x3 SVD");
        double m[9], U[9], V[9], S[3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) m[i * 3 + j] = static_cast<double>(M(i, j));
        orc::linalg::svd3(m, U, S, V);
        for (int i = 0; i < 3; ++i) {
            sv_(i) = static_cast<T>(S[i]);
            for (int j = 0; j < 3; ++j) {
                u_(i, j) = static_cast<T>(U[i * 3 + j]);
                v_(i, j) = static_cast<T>(V[i * 3 + j]);
            }
        }
    }
    const MatrixType& matrixU() const { return u_; }
    const MatrixType& matrixV() const { return v_; }
    const Matrix<T, 3, 1>& singularValues() const { return sv_; }

private:
    MatrixType u_, v_;
    Matrix<T, 3, 1> sv_;
};

}  // namespace Eigen
