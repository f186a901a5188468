/* A project-written stand-in for the part of Eigen that the reference's
 * src/solnoutclass.hpp uses, so that its Parasitics and SolverDataBase code
 * (network-parameter conversion, the output writers, the .sim_input reader)
 * compiles here unmodified.  Eigen itself is not in the image.
 *
 * Dense matrices (row-major storage whatever the options), column vectors,
 * dynamic diagonal matrices, triplets and a CSR sparse matrix with an inner
 * iterator.  The arithmetic is plain: products as row-by-column sums in
 * index order, inverse() by Gauss-Jordan elimination with partial pivoting,
 * isApprox as Eigen documents it (squared Frobenius norm of the difference
 * within prec^2 times the smaller squared norm).  Results therefore agree
 * with Eigen's to rounding, not bit for bit.
 * TEST INFRASTRUCTURE ONLY. */
#ifndef G2P_EIGEN_STANDIN_HPP
#define G2P_EIGEN_STANDIN_HPP

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <type_traits>
#include <vector>

namespace Eigen {

enum { Dynamic = -1 };
enum { ColMajor = 0, RowMajor = 1 };
enum { Lower = 1, Upper = 2 };

namespace standin {
template <class T> struct real_of { typedef T type; };
template <class T> struct real_of<std::complex<T>> { typedef T type; };
template <class T> double abs2(const T &v) { return (double)std::norm(std::complex<double>(v)); }
}  // namespace standin

template <class T, int O = ColMajor, class I = int> class SparseMatrix;

template <class T, int R = Dynamic, int C = Dynamic, int O = (R == 1 && C != 1) ? RowMajor : ColMajor>
class Matrix {
public:
    typedef T Scalar;
    std::vector<T> d;      // row-major
    long r = 0, c = 0;

    Matrix() {
        if (R > 0 && C > 0) resize(R, C);
    }
    Matrix(long rows, long cols) { resize(rows, cols); }
    template <class I, class = typename std::enable_if<std::is_integral<I>::value>::type>
    explicit Matrix(I n) {
        if (C == 1) resize((long)n, 1);
        else resize(1, (long)n);
    }
    template <class U, int R2, int C2, int O2>
    Matrix(const Matrix<U, R2, C2, O2> &o) { assign(o); }
    template <class U, int R2, int C2, int O2>
    Matrix &operator=(const Matrix<U, R2, C2, O2> &o) { assign(o); return *this; }

    template <class U, int R2, int C2, int O2>
    void assign(const Matrix<U, R2, C2, O2> &o) {
        r = o.r; c = o.c;
        d.assign(o.d.size(), T(0));
        for (size_t i = 0; i < o.d.size(); i++) d[i] = T(o.d[i]);
    }

    long rows() const { return r; }
    long cols() const { return c; }
    long size() const { return r * c; }
    long outerSize() const { return r; }
    long innerSize() const { return c; }
    T &operator[](long i) { return d[(size_t)i]; }
    const T &operator[](long i) const { return d[(size_t)i]; }
    template <class U, int O2, class I2>
    Matrix &operator=(const SparseMatrix<U, O2, I2> &sp);
    // rowwise().sum(): the row sums as a column vector
    struct RowwiseView {
        const Matrix &m;
        Matrix<T, Dynamic, 1> sum() const {
            Matrix<T, Dynamic, 1> v(m.r, 1);
            for (long i = 0; i < m.r; i++) {
                T s = T(0);
                for (long j = 0; j < m.c; j++) s += m(i, j);
                v(i) = s;
            }
            return v;
        }
    };
    RowwiseView rowwise() const { return RowwiseView{*this}; }
    Matrix<typename standin::real_of<T>::type, R, C, O> real() const {
        Matrix<typename standin::real_of<T>::type, R, C, O> t;
        t.r = r; t.c = c; t.d.resize(d.size());
        for (size_t i = 0; i < d.size(); i++) t.d[i] = std::real(d[i]);
        return t;
    }
    Matrix<typename standin::real_of<T>::type, R, C, O> imag() const {
        Matrix<typename standin::real_of<T>::type, R, C, O> t;
        t.r = r; t.c = c; t.d.resize(d.size());
        for (size_t i = 0; i < d.size(); i++) t.d[i] = std::imag(d[i]);
        return t;
    }
    void resize(long rows, long cols) { r = rows; c = cols; d.assign((size_t)(rows * cols), T(0)); }
    void resize(long n) { if (C == 1) resize(n, 1); else resize(1, n); }
    void setZero() { std::fill(d.begin(), d.end(), T(0)); }
    void setZero(long rows, long cols) { resize(rows, cols); }
    T &operator()(long i, long j) { return d[(size_t)(i * c + j)]; }
    const T &operator()(long i, long j) const { return d[(size_t)(i * c + j)]; }
    T &operator()(long i) { return d[(size_t)i]; }
    const T &operator()(long i) const { return d[(size_t)i]; }
    T &coeffRef(long i, long j) { return (*this)(i, j); }
    T coeff(long i, long j) const { return (*this)(i, j); }

    static Matrix Identity(long rows, long cols) {
        Matrix m(rows, cols);
        for (long i = 0; i < std::min(rows, cols); i++) m(i, i) = T(1);
        return m;
    }
    static Matrix Zero(long rows, long cols) { return Matrix(rows, cols); }
    static Matrix Zero(long n) { Matrix m; m.resize(n); return m; }

    Matrix transpose() const {
        Matrix t(c, r);
        for (long i = 0; i < r; i++)
            for (long j = 0; j < c; j++) t(j, i) = (*this)(i, j);
        return t;
    }
    Matrix conjugate() const {
        Matrix t(*this);
        for (auto &v : t.d) v = conj_of(v);
        return t;
    }
    Matrix adjoint() const { return transpose().conjugate(); }
    // diagonal as a column vector (read); DiagonalMatrix has the writable one
    Matrix<T, Dynamic, 1> diagonal() const {
        Matrix<T, Dynamic, 1> v(std::min(r, c), 1);
        for (long i = 0; i < v.r; i++) v(i) = (*this)(i, i);
        return v;
    }
    T sum() const {
        T s = T(0);
        for (const auto &v : d) s += v;
        return s;
    }
    double squaredNorm() const {
        double s = 0;
        for (const auto &v : d) s += standin::abs2(v);
        return s;
    }
    double norm() const { return std::sqrt(squaredNorm()); }
    template <int Mode>
    Matrix triangularView() const {
        Matrix t(r, c);
        for (long i = 0; i < r; i++)
            for (long j = 0; j < c; j++)
                if ((Mode == Upper && j >= i) || (Mode == Lower && j <= i)) t(i, j) = (*this)(i, j);
        return t;
    }
    template <class U, int R2, int C2, int O2>
    bool isApprox(const Matrix<U, R2, C2, O2> &o, double prec = 1e-12) const {
        double dn = 0;
        for (size_t i = 0; i < d.size(); i++) dn += standin::abs2(std::complex<double>(d[i]) - std::complex<double>(o.d[i]));
        return dn <= prec * prec * std::min(squaredNorm(), o.squaredNorm());
    }
    // Gauss-Jordan elimination with partial pivoting
    Matrix inverse() const {
        const long n = r;
        Matrix a(*this), inv = Identity(n, n);
        for (long k = 0; k < n; k++) {
            long p = k;
            double best = std::abs(std::complex<double>(a(k, k)));
            for (long i = k + 1; i < n; i++) {
                const double v = std::abs(std::complex<double>(a(i, k)));
                if (v > best) { best = v; p = i; }
            }
            if (p != k)
                for (long j = 0; j < n; j++) { std::swap(a(k, j), a(p, j)); std::swap(inv(k, j), inv(p, j)); }
            const T piv = a(k, k);
            for (long j = 0; j < n; j++) { a(k, j) /= piv; inv(k, j) /= piv; }
            for (long i = 0; i < n; i++) {
                if (i == k) continue;
                const T f = a(i, k);
                if (f == T(0)) continue;
                for (long j = 0; j < n; j++) { a(i, j) -= f * a(k, j); inv(i, j) -= f * inv(k, j); }
            }
        }
        return inv;
    }

    Matrix operator-() const { Matrix t(*this); for (auto &v : t.d) v = -v; return t; }
    Matrix &operator+=(const Matrix &o) { for (size_t i = 0; i < d.size(); i++) d[i] += o.d[i]; return *this; }
    Matrix &operator-=(const Matrix &o) { for (size_t i = 0; i < d.size(); i++) d[i] -= o.d[i]; return *this; }
    Matrix operator+(const Matrix &o) const { Matrix t(*this); t += o; return t; }
    Matrix operator-(const Matrix &o) const { Matrix t(*this); t -= o; return t; }
    template <int R2, int C2, int O2>
    Matrix<T, Dynamic, Dynamic, RowMajor> operator*(const Matrix<T, R2, C2, O2> &o) const {
        Matrix<T, Dynamic, Dynamic, RowMajor> t(r, o.c);
        for (long i = 0; i < r; i++)
            for (long j = 0; j < o.c; j++) {
                T s = T(0);
                for (long k = 0; k < c; k++) s += (*this)(i, k) * o(k, j);
                t(i, j) = s;
            }
        return t;
    }
    template <class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    Matrix operator*(S s) const { Matrix t(*this); for (auto &v : t.d) v *= T(s); return t; }
    Matrix operator*(const std::complex<double> &s) const { Matrix t(*this); for (auto &v : t.d) v = v * T(s); return t; }
    template <class S>
    Matrix operator/(S s) const { Matrix t(*this); for (auto &v : t.d) v /= T(s); return t; }
    template <class S>
    Matrix &operator*=(S s) { for (auto &v : d) v *= T(s); return *this; }

private:
    template <class V> static V conj_of(const V &v) { return v; }
    template <class V> static std::complex<V> conj_of(const std::complex<V> &v) { return std::conj(v); }
};

template <class S, class T, int R, int C, int O, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
Matrix<T, R, C, O> operator*(S s, const Matrix<T, R, C, O> &m) { return m * s; }

// complex scalar times a real or complex matrix: a complex matrix
template <class T, int R, int C, int O>
Matrix<std::complex<double>, R, C, O> operator*(const std::complex<double> &s, const Matrix<T, R, C, O> &m) {
    Matrix<std::complex<double>, R, C, O> t;
    t.r = m.r; t.c = m.c; t.d.resize(m.d.size());
    for (size_t i = 0; i < m.d.size(); i++) t.d[i] = s * std::complex<double>(m.d[i]);
    return t;
}
// real + complex matrix: a complex matrix
template <int R, int C, int O, int R2, int C2, int O2>
Matrix<std::complex<double>, R, C, O> operator+(const Matrix<double, R, C, O> &a,
                                                 const Matrix<std::complex<double>, R2, C2, O2> &b) {
    Matrix<std::complex<double>, R, C, O> t;
    t.r = a.r; t.c = a.c; t.d.resize(a.d.size());
    for (size_t i = 0; i < a.d.size(); i++) t.d[i] = std::complex<double>(a.d[i]) + b.d[i];
    return t;
}

typedef Matrix<double, Dynamic, 1> VectorXd;
typedef Matrix<std::complex<double>, Dynamic, 1> VectorXcd;
typedef Matrix<double, Dynamic, Dynamic> MatrixXd;
typedef Matrix<std::complex<double>, Dynamic, Dynamic> MatrixXcd;

template <class T, int N = Dynamic>
class DiagonalMatrix {
public:
    Matrix<T, Dynamic, 1> v;
    DiagonalMatrix() {}
    explicit DiagonalMatrix(long n) : v(n, 1) {}
    Matrix<T, Dynamic, 1> &diagonal() { return v; }
    const Matrix<T, Dynamic, 1> &diagonal() const { return v; }
    long rows() const { return v.r; }
    long cols() const { return v.r; }
};

template <class T, int N, int R, int C, int O>
Matrix<T, Dynamic, Dynamic, RowMajor> operator*(const DiagonalMatrix<T, N> &D, const Matrix<T, R, C, O> &m) {
    Matrix<T, Dynamic, Dynamic, RowMajor> t(m.r, m.c);
    for (long i = 0; i < m.r; i++)
        for (long j = 0; j < m.c; j++) t(i, j) = D.v(i) * m(i, j);
    return t;
}
template <class T, int N, int R, int C, int O>
Matrix<T, Dynamic, Dynamic, RowMajor> operator*(const Matrix<T, R, C, O> &m, const DiagonalMatrix<T, N> &D) {
    Matrix<T, Dynamic, Dynamic, RowMajor> t(m.r, m.c);
    for (long i = 0; i < m.r; i++)
        for (long j = 0; j < m.c; j++) t(i, j) = m(i, j) * D.v(j);
    return t;
}

template <class T, class I = int>
class Triplet {
public:
    Triplet() : r_(0), c_(0), v_(0) {}
    Triplet(const I &r, const I &c, const T &v = T(0)) : r_(r), c_(c), v_(v) {}
    const I &row() const { return r_; }
    const I &col() const { return c_; }
    const T &value() const { return v_; }
private:
    I r_, c_;
    T v_;
};

// CSR sparse matrix (rows are the outer dimension whatever the options)
template <class T, int O, class I>
class SparseMatrix {
public:
    typedef T Scalar;
    long r = 0, c = 0;
    std::vector<long> ptr{0};
    std::vector<long> idx;
    std::vector<T> val;

    SparseMatrix() {}
    SparseMatrix(long rows, long cols) : r(rows), c(cols), ptr((size_t)rows + 1, 0) {}
    long rows() const { return r; }
    long cols() const { return c; }
    long outerSize() const { return r; }
    long innerSize() const { return c; }
    long nonZeros() const { return (long)val.size(); }
    void resize(long rows, long cols) { r = rows; c = cols; ptr.assign((size_t)rows + 1, 0); idx.clear(); val.clear(); }
    void setZero() { resize(r, c); }
    void makeCompressed() {}
    void reserve(long) {}
    template <class It>
    void setFromTriplets(It first, It last) {
        std::vector<std::vector<std::pair<long, T>>> rowsv((size_t)r);
        for (It it = first; it != last; ++it) rowsv[(size_t)it->row()].push_back({(long)it->col(), it->value()});
        ptr.assign((size_t)r + 1, 0);
        idx.clear(); val.clear();
        for (long i = 0; i < r; i++) {
            auto &rv = rowsv[(size_t)i];
            std::stable_sort(rv.begin(), rv.end(), [](const std::pair<long, T> &a, const std::pair<long, T> &b) { return a.first < b.first; });
            for (size_t k = 0; k < rv.size(); k++) {
                if (k > 0 && rv[k].first == rv[k - 1].first) { val.back() += rv[k].second; continue; }
                idx.push_back(rv[k].first);
                val.push_back(rv[k].second);
            }
            ptr[(size_t)i + 1] = (long)val.size();
        }
    }
    T coeff(long i, long j) const {
        for (long q = ptr[(size_t)i]; q < ptr[(size_t)i + 1]; q++) if (idx[(size_t)q] == j) return val[(size_t)q];
        return T(0);
    }
    T &coeffRef(long i, long j) {
        for (long q = ptr[(size_t)i]; q < ptr[(size_t)i + 1]; q++) if (idx[(size_t)q] == j) return val[(size_t)q];
        // insert keeping columns sorted
        long q = ptr[(size_t)i];
        while (q < ptr[(size_t)i + 1] && idx[(size_t)q] < j) q++;
        idx.insert(idx.begin() + q, j);
        val.insert(val.begin() + q, T(0));
        for (long k = i + 1; k <= r; k++) ptr[(size_t)k]++;
        return val[(size_t)q];
    }
    template <class F>
    void prune(const F &keep) {
        std::vector<long> np((size_t)r + 1, 0), ni;
        std::vector<T> nv;
        for (long i = 0; i < r; i++) {
            for (long q = ptr[(size_t)i]; q < ptr[(size_t)i + 1]; q++)
                if (keep(i, idx[(size_t)q], val[(size_t)q])) { ni.push_back(idx[(size_t)q]); nv.push_back(val[(size_t)q]); }
            np[(size_t)i + 1] = (long)nv.size();
        }
        ptr = np; idx = ni; val = nv;
    }

    class InnerIterator {
    public:
        InnerIterator(const SparseMatrix &m, long outer) : m_(m), o_(outer), q_(m.ptr[(size_t)outer]) {}
        InnerIterator &operator++() { q_++; return *this; }
        explicit operator bool() const { return q_ < m_.ptr[(size_t)o_ + 1]; }
        long row() const { return o_; }
        long col() const { return m_.idx[(size_t)q_]; }
        long index() const { return m_.idx[(size_t)q_]; }
        long outer() const { return o_; }
        const T &value() const { return m_.val[(size_t)q_]; }
    private:
        const SparseMatrix &m_;
        long o_, q_;
    };
};

template <class T, int R, int C, int O>
template <class U, int O2, class I2>
Matrix<T, R, C, O> &Matrix<T, R, C, O>::operator=(const SparseMatrix<U, O2, I2> &sp) {
    resize(sp.r, sp.c);
    for (long i = 0; i < sp.r; i++)
        for (long q = sp.ptr[(size_t)i]; q < sp.ptr[(size_t)i + 1]; q++) (*this)(i, sp.idx[(size_t)q]) = T(sp.val[(size_t)q]);
    return *this;
}

}  // namespace Eigen

#endif
