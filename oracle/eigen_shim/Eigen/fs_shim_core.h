// Project-written stand-in for the small part of the Eigen 3 API that the
// Fluid_Simulation reference uses.  It exists only so that the reference's own
// sources (src/FluidSolver.cpp, src/FluidDomain.cpp, src/MacGrid.cpp,
// src/MarkerParticleSet.cpp, src/LevelSet.cpp) compile unmodified for the
// oracle build; it is test infrastructure, never part of the product.
//
// Eigen itself is third-party, not vendored in the reference, and its version
// is unpinned there (CMakeLists.txt:15-17 asks pkg-config for "eigen3").  The
// surface used by the reference is:
//   MathDefinitions.h:10,13        Eigen::VectorXd / Eigen::VectorXf
//   FluidSolver.h:114,116          ConjugateGradient<SparseMatrix<float>>, SparseMatrix<float>
//   FluidSolver.cpp:81             ConjugateGradient::setMaxIterations
//   FluidSolver.cpp:363-366        SparseMatrix::resize / reserve, VectorXi::Constant, VectorX(n)
//   FluidSolver.cpp:381-413        SparseMatrix::insert(row, col) = value, b[idx] = ...
//   FluidSolver.cpp:423-425        VectorX x(n); cg.compute(A); x = cg.solve(b)
//   FluidSolver.cpp:455-460        x(idx)
//
// The conjugate-gradient solver below is the published Jacobi-preconditioned
// CG algorithm (Hestenes-Stiefel with a diagonal preconditioner, zero initial
// guess, stop when ||r||^2 < tol^2 ||b||^2 or after maxIterations updates;
// default tolerance = machine epsilon of the scalar, as Eigen documents for
// ConjugateGradient), written from the textbook, not from Eigen's source.
// Its floating-point discipline is fixed so that the CPU restatement
// (oracle/fs_oracle.c) and the GPU path can reproduce it bit for bit:
//   * vectors and the SpMV are in the scalar type (float), with every product
//     and sum rounded separately (build with -ffp-contract=off);
//   * dot products and norms sum their terms along the fixed "32-ary
//     stride-halving tree" of fs_rsum32() below, in one of two precisions
//     (fs_cg_precision()):
//       FS_CG_FLOAT (default, the reference's own precision: Eigen's
//         VectorXf dot products are float) -- float products, float tree,
//         alpha, beta and the threshold tol^2 ||b||^2 in float;
//       FS_CG_DOUBLE -- exact float*float products summed in double, alpha
//         and beta formed in double and rounded once to float;
// The SpMV walks the self-adjoint matrix built from the lower triangle
// (Eigen's default UpLo = Lower) and sums the entries of each row in
// ascending column order, starting from +0.
#ifndef FS_EIGEN_SHIM_CORE_H
#define FS_EIGEN_SHIM_CORE_H

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstddef>
#include <limits>
#include <utility>
#include <vector>

namespace Eigen {

typedef std::ptrdiff_t Index;

// Sum of n doubles by the fixed 32-ary tree: split into groups of 32
// consecutive values (zero padded), reduce each group by the stride-halving
// tree (s = 16, 8, 4, 2, 1: a[l] += a[l + s]), and repeat on the group
// results until one value is left.  Destroys its input.
template <typename T>
inline T fs_rsum32(std::vector<T>& a, Index n)
{
    if (n <= 0) return 0.0;
    while (n > 1) {
        Index groups = (n + 31) / 32;
        for (Index g = 0; g < groups; ++g) {
            T t[32];
            for (int l = 0; l < 32; ++l) {
                Index k = g * 32 + l;
                t[l] = k < n ? a[k] : T(0);
            }
            for (int s = 16; s >= 1; s >>= 1)
                for (int l = 0; l < s; ++l) t[l] = t[l] + t[l + s];
            a[g] = t[0];
        }
        n = groups;
    }
    return a[0];
}

template <typename T>
class DenseVector
{
public:
    DenseVector() {}
    explicit DenseVector(Index n) : d_(static_cast<size_t>(n), T(0)) {}
    static DenseVector Constant(Index n, const T& v)
    {
        DenseVector r(n);
        std::fill(r.d_.begin(), r.d_.end(), v);
        return r;
    }
    Index size() const { return static_cast<Index>(d_.size()); }
    void resize(Index n) { d_.assign(static_cast<size_t>(n), T(0)); }
    T& operator[](Index i) { return d_[static_cast<size_t>(i)]; }
    const T& operator[](Index i) const { return d_[static_cast<size_t>(i)]; }
    T& operator()(Index i) { return d_[static_cast<size_t>(i)]; }
    const T& operator()(Index i) const { return d_[static_cast<size_t>(i)]; }
    T* data() { return d_.data(); }
    const T* data() const { return d_.data(); }

private:
    std::vector<T> d_;
};

typedef DenseVector<float> VectorXf;
typedef DenseVector<double> VectorXd;
typedef DenseVector<int> VectorXi;

// Minimal sparse matrix: entries are collected by insert() and frozen into a
// symmetric row view (lower triangle mirrored) when a solver compute()s it.
template <typename T>
class SparseMatrix
{
public:
    typedef T Scalar;
    SparseMatrix() : rows_(0), cols_(0) {}
    void resize(Index rows, Index cols)
    {
        rows_ = rows;
        cols_ = cols;
        entries_.clear();
    }
    template <typename Sizes>
    void reserve(const Sizes&)
    {
        // A capacity hint in Eigen; nothing to do here.  (The reference passes
        // VectorXi::Constant(5, n), i.e. a 5-element vector of value n.)
    }
    T& insert(Index row, Index col)
    {
        entries_.push_back(Entry{row, col, T(0)});
        return entries_.back().value;
    }
    Index rows() const { return rows_; }
    Index cols() const { return cols_; }

    struct Entry
    {
        Index row, col;
        T value;
    };
    const std::vector<Entry>& entries() const { return entries_; }

private:
    Index rows_, cols_;
    // std::vector of entries: insert() returns a reference that the caller
    // writes through immediately (FluidSolver.cpp:381-410), before the next
    // insert can reallocate.
    std::vector<Entry> entries_;
};

enum { FS_CG_FLOAT = 0, FS_CG_DOUBLE = 1 };
inline int& fs_cg_precision()
{
    static int p = FS_CG_FLOAT;
    return p;
}

struct FsCgRecord
{
    // Last solve of any ConjugateGradient in this process, kept for the
    // oracle harness (the reference keeps the pressure only in a local).
    std::vector<double> solution;
    Index iterations = 0;
    double error = 0.0;
};
inline FsCgRecord& fs_cg_record()
{
    static FsCgRecord r;
    return r;
}

template <typename MatrixType>
class ConjugateGradient
{
public:
    typedef typename MatrixType::Scalar Scalar;

    ConjugateGradient()
        : max_iter_(-1), tol_(std::numeric_limits<Scalar>::epsilon()), iters_(0), error_(0.0), n_(0) {}

    void setMaxIterations(Index n) { max_iter_ = n; }
    void setTolerance(double tol) { tol_ = tol; }
    Index maxIterations() const { return max_iter_ < 0 ? 2 * n_ : max_iter_; }
    double tolerance() const { return tol_; }
    Index iterations() const { return iters_; }
    double error() const { return error_; }

    ConjugateGradient& compute(const MatrixType& A)
    {
        n_ = A.rows();
        rows_.assign(static_cast<size_t>(n_), std::vector<std::pair<Index, Scalar>>());
        diag_.assign(static_cast<size_t>(n_), Scalar(0));
        for (const auto& e : A.entries()) {
            if (e.row > e.col) {
                rows_[static_cast<size_t>(e.row)].push_back({e.col, e.value});
                rows_[static_cast<size_t>(e.col)].push_back({e.row, e.value});
            } else if (e.row == e.col) {
                rows_[static_cast<size_t>(e.row)].push_back({e.col, e.value});
                diag_[static_cast<size_t>(e.row)] = e.value;
            }
        }
        for (auto& r : rows_)
            std::sort(r.begin(), r.end(),
                      [](const std::pair<Index, Scalar>& a, const std::pair<Index, Scalar>& b) {
                          return a.first < b.first;
                      });
        inv_diag_.resize(static_cast<size_t>(n_));
        for (Index k = 0; k < n_; ++k) {
            Scalar d = diag_[static_cast<size_t>(k)];
            inv_diag_[static_cast<size_t>(k)] = d != Scalar(0) ? Scalar(1) / d : Scalar(1);
        }
        return *this;
    }

    template <typename Rhs>
    Rhs solve(const Rhs& b)
    {
        if (fs_cg_precision() == FS_CG_DOUBLE) return solve_t<Rhs, double>(b);
        return solve_t<Rhs, float>(b);
    }

    // R: accumulation type of the dot products (float or double).
    template <typename Rhs, typename R>
    Rhs solve_t(const Rhs& b)
    {
        const Index n = n_;
        Rhs x(n);
        std::vector<R> scratch(static_cast<size_t>(n > 0 ? n : 1));
        auto dot = [&](const std::vector<Scalar>& a, const std::vector<Scalar>& c) {
            for (Index k = 0; k < n; ++k)
                scratch[static_cast<size_t>(k)] =
                    static_cast<R>(a[static_cast<size_t>(k)]) * static_cast<R>(c[static_cast<size_t>(k)]);
            return fs_rsum32<R>(scratch, n);
        };
        std::vector<Scalar> r(static_cast<size_t>(n)), p(static_cast<size_t>(n)),
            q(static_cast<size_t>(n)), z(static_cast<size_t>(n)), xv(static_cast<size_t>(n), Scalar(0));
        for (Index k = 0; k < n; ++k) r[static_cast<size_t>(k)] = b[k];

        iters_ = 0;
        error_ = 0.0;
        const R bb = dot(r, r);
        if (bb == R(0)) {
            record(xv);
            return x;
        }
        const R tol = static_cast<R>(tol_);
        R thr = tol * tol;
        thr = thr * bb;
        if (thr < std::numeric_limits<R>::min()) thr = std::numeric_limits<R>::min();
        R rr = bb;
        if (rr < thr) {
            error_ = std::sqrt(static_cast<double>(rr) / static_cast<double>(bb));
            record(xv);
            return x;
        }
        for (Index k = 0; k < n; ++k)
            p[static_cast<size_t>(k)] = inv_diag_[static_cast<size_t>(k)] * r[static_cast<size_t>(k)];
        R rz = dot(r, p);
        const Index maxit = maxIterations();
        for (Index it = 1; it <= maxit; ++it) {
            for (Index k = 0; k < n; ++k) {
                Scalar acc = Scalar(0);
                for (const auto& e : rows_[static_cast<size_t>(k)]) {
                    Scalar t = e.second * p[static_cast<size_t>(e.first)];
                    acc = acc + t;
                }
                q[static_cast<size_t>(k)] = acc;
            }
            const R pq = dot(p, q);
            const Scalar alpha = static_cast<Scalar>(rz / pq);
            for (Index k = 0; k < n; ++k) {
                Scalar ap = alpha * p[static_cast<size_t>(k)];
                xv[static_cast<size_t>(k)] = xv[static_cast<size_t>(k)] + ap;
                Scalar aq = alpha * q[static_cast<size_t>(k)];
                r[static_cast<size_t>(k)] = r[static_cast<size_t>(k)] - aq;
            }
            rr = dot(r, r);
            iters_ = it;
            if (rr < thr) break;
            for (Index k = 0; k < n; ++k)
                z[static_cast<size_t>(k)] = inv_diag_[static_cast<size_t>(k)] * r[static_cast<size_t>(k)];
            const R rz_new = dot(r, z);
            const Scalar beta = static_cast<Scalar>(rz_new / rz);
            rz = rz_new;
            for (Index k = 0; k < n; ++k) {
                Scalar bp = beta * p[static_cast<size_t>(k)];
                p[static_cast<size_t>(k)] = z[static_cast<size_t>(k)] + bp;
            }
        }
        error_ = std::sqrt(static_cast<double>(rr) / static_cast<double>(bb));
        for (Index k = 0; k < n; ++k) x[k] = xv[static_cast<size_t>(k)];
        record(xv);
        return x;
    }

private:
    void record(const std::vector<Scalar>& xv)
    {
        FsCgRecord& rec = fs_cg_record();
        rec.solution.assign(xv.begin(), xv.end());
        rec.iterations = iters_;
        rec.error = error_;
    }

    Index max_iter_;
    double tol_;
    Index iters_;
    double error_;
    Index n_;
    std::vector<std::vector<std::pair<Index, Scalar>>> rows_;
    std::vector<Scalar> diag_, inv_diag_;
};

}  // namespace Eigen

#endif
