// ShimDense.h — the subset of Eigen's dense API that the reference's simulation code uses,
// written for this project from Eigen's documented semantics (no Eigen source is used).
//
// TEST INFRASTRUCTURE ONLY.  It lets the unmodified reference sources (LevelSetLiquid and
// the files it needs) compile into oracle/_ref, the reference binary the CPU port and the
// GPU kernels are checked against.  Fixed-size vectors and matrices are plain column-major
// arrays (so std::vector<Vector3d> has the layout Eigen gives it: 3 doubles per element, a
// 3x3 matrix 9 doubles column by column).  Every operation is evaluated eagerly, in index
// order; where Eigen's vectorised reductions add in another order the two differ by
// rounding only.  Matrix and Array are one class with a kind flag: Array multiplies and
// compares element by element, Matrix multiplies as matrices.
#pragma once

#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <initializer_list>
#include <limits>
#include <ostream>
#include <type_traits>
#include <vector>

namespace Eigen {

using Index = std::ptrdiff_t;
constexpr int Dynamic = -1;
constexpr int Infinity = -1;
enum StorageOptions { ColMajor = 0, RowMajor = 0x1, AutoAlign = 0, DontAlign = 0x2 };
enum AlignmentType { Unaligned = 0, Aligned8 = 8, Aligned16 = 16, Aligned32 = 32, Aligned64 = 64, Aligned128 = 128, AlignedMax = 16, Aligned = 16 };
enum UpLoType { Lower = 0x1, Upper = 0x2 };
enum ComputationInfo { Success = 0, NumericalIssue = 1, NoConvergence = 2, InvalidInput = 3 };
enum { StreamPrecision = -1, FullPrecision = -2 };

namespace shim {
template <typename S, int R, int C> struct Storage {
	S v[R * C] = {};
	S *data() { return v; }
	const S *data() const { return v; }
	static constexpr Index rows() { return R; }
	static constexpr Index cols() { return C; }
	void resize(Index r, Index c) { assert(r == R && c == C); (void)r; (void)c; }
};
template <typename S, int C> struct Storage<S, Dynamic, C> {
	std::vector<S> v;
	Index r = 0;
	S *data() { return v.data(); }
	const S *data() const { return v.data(); }
	Index rows() const { return r; }
	static constexpr Index cols() { return C; }
	void resize(Index rr, Index c) { assert(c == C); (void)c; r = rr; v.assign(size_t(rr) * C, S(0)); }
};
template <typename S> struct Storage<S, Dynamic, Dynamic> {
	std::vector<S> v;
	Index r = 0, c = 0;
	S *data() { return v.data(); }
	const S *data() const { return v.data(); }
	Index rows() const { return r; }
	Index cols() const { return c; }
	void resize(Index rr, Index cc) { r = rr; c = cc; v.assign(size_t(rr) * size_t(cc), S(0)); }
};
template <typename T> inline T sgn(T a) { return T((T(0) < a) - (a < T(0))); }
}  // namespace shim

// Options and maximum sizes are carried so that Matrix and Array alias Dense with every
// parameter used: an alias that drops parameters is not interchangeable with its expansion
// in dependent declarations, and the reference spells one type both ways.
template <typename S, int R, int C, int O, int MR, int MC, bool IsArray> class Dense;
template <typename S, int R, int C, int O = 0, int MR = R, int MC = C> using Matrix = Dense<S, R, C, O, MR, MC, false>;
template <typename S, int R, int C, int O = 0, int MR = R, int MC = C> using Array = Dense<S, R, C, O, MR, MC, true>;
template <typename S, int R, int C, bool IsArray> using DenseOf = Dense<S, R, C, 0, R, C, IsArray>;

struct IOFormat {
	int precision;
	IOFormat(int p = StreamPrecision, int = 0, const char * = " ", const char * = "\n", const char * = "", const char * = "",
	         const char * = "", const char * = "") : precision(p) { }
};

// A writable view of column j (contiguous) or row i (stride R) of a matrix.
template <typename V> class LineRef {
public:
	using Scalar = typename V::Scalar;
	LineRef(Scalar *p, Index stride) : _p(p), _stride(stride) { }
	Scalar &operator[](Index i) { return _p[i * _stride]; }
	Scalar operator[](Index i) const { return _p[i * _stride]; }
	Scalar &operator()(Index i) { return _p[i * _stride]; }
	Scalar operator()(Index i) const { return _p[i * _stride]; }
	static constexpr Index size() { return V::SizeAtCompileTime; }
	V eval() const { V out; for (Index i = 0; i < size(); i++) out[i] = (*this)[i]; return out; }
	operator V() const { return eval(); }
	LineRef &operator=(const V &o) { for (Index i = 0; i < size(); i++) (*this)[i] = o[i]; return *this; }
	LineRef &operator=(const LineRef &o) { return *this = o.eval(); }
	LineRef &operator+=(const V &o) { for (Index i = 0; i < size(); i++) (*this)[i] += o[i]; return *this; }
	LineRef &operator-=(const V &o) { for (Index i = 0; i < size(); i++) (*this)[i] -= o[i]; return *this; }
	LineRef &operator*=(Scalar s) { for (Index i = 0; i < size(); i++) (*this)[i] *= s; return *this; }
	Scalar norm() const { return eval().norm(); }
	Scalar squaredNorm() const { return eval().squaredNorm(); }
	V normalized() const { return eval().normalized(); }
	Scalar dot(const V &o) const { return eval().dot(o); }
	auto transpose() const { return eval().transpose(); }
	auto array() const { return eval().array(); }
	Scalar sum() const { return eval().sum(); }
	Scalar maxCoeff() const { return eval().maxCoeff(); }
private:
	Scalar *_p;
	Index _stride;
};

template <typename S, int R, int C, int O, int MR, int MC, bool IsArray>
class Dense {
public:
	using Scalar = S;
	using RealScalar = S;
	using PlainObject = Dense;
	static constexpr int RowsAtCompileTime = R, ColsAtCompileTime = C;
	static constexpr int SizeAtCompileTime = (R == Dynamic || C == Dynamic) ? Dynamic : R * C;
	static constexpr bool IsVectorAtCompileTime = R == 1 || C == 1;
	static constexpr bool IsFixed = SizeAtCompileTime != Dynamic;

	shim::Storage<S, R, C> st;

	Dense() = default;
	Dense(const Dense &) = default;
	Dense &operator=(const Dense &) = default;
	template <typename T, int R2, int C2, int O2, int MR2, int MC2, bool A2> friend class Dense;
	// dynamic vectors and matrices: sizes.  A fixed-size object given an integer (Eigen reads
	// it as the size and leaves the coefficients unset, as in Zero() of a matrix whose
	// scalar is itself a vector, SGridBasedData.h:23) is zero-filled.
	template <typename I, std::enable_if_t<std::is_integral_v<I>, int> = 0>
	explicit Dense(I n) {
		if constexpr (!IsFixed) { if constexpr (C == Dynamic) st.resize(Index(n), 1); else st.resize(Index(n), C); }
	}
	template <typename I, typename J, std::enable_if_t<std::is_integral_v<I> && std::is_integral_v<J> && !IsFixed, int> = 0>
	Dense(I r, J c) { st.resize(Index(r), Index(c)); }
	// fixed vectors: coefficients
	template <typename A0, typename A1, std::enable_if_t<std::is_arithmetic_v<A0> && std::is_arithmetic_v<A1> && IsFixed, int> = 0>
	Dense(A0 a, A1 b) { static_assert(SizeAtCompileTime == 2); st.v[0] = S(a); st.v[1] = S(b); }
	template <typename A0, typename A1, typename A2, std::enable_if_t<std::is_arithmetic_v<A0> && IsFixed, int> = 0>
	Dense(A0 a, A1 b, A2 c) { static_assert(SizeAtCompileTime == 3); st.v[0] = S(a); st.v[1] = S(b); st.v[2] = S(c); }
	template <typename A0, typename A1, typename A2, typename A3, std::enable_if_t<std::is_arithmetic_v<A0> && IsFixed, int> = 0>
	Dense(A0 a, A1 b, A2 c, A3 d) { static_assert(SizeAtCompileTime == 4); st.v[0] = S(a); st.v[1] = S(b); st.v[2] = S(c); st.v[3] = S(d); }
	// the other kind (matrix <-> array) of the same shape and scalar
	Dense(const Dense<S, R, C, O, MR, MC, !IsArray> &o) { st = o.st; }

	// sizes and coefficients
	Index rows() const { return st.rows(); }
	Index cols() const { return st.cols(); }
	Index size() const { return rows() * cols(); }
	S *data() { return st.data(); }
	const S *data() const { return st.data(); }
	void resize(Index n) { if constexpr (C == Dynamic) st.resize(n, 1); else st.resize(n / C, C); }
	void resize(Index r, Index c) { st.resize(r, c); }
	S &operator[](Index i) { return data()[i]; }
	const S &operator[](Index i) const { return data()[i]; }
	S &operator()(Index i) { return data()[i]; }
	const S &operator()(Index i) const { return data()[i]; }
	S &operator()(Index r, Index c) { return data()[r + c * rows()]; }
	const S &operator()(Index r, Index c) const { return data()[r + c * rows()]; }
	S value() const { static_assert(SizeAtCompileTime == 1); return data()[0]; }
	S coeff(Index i) const { return data()[i]; }
	S &coeffRef(Index i) { return data()[i]; }
	S &x() { return data()[0]; }
	S &y() { return data()[1]; }
	S &z() { return data()[2]; }
	S &w() { return data()[3]; }
	const S &x() const { return data()[0]; }
	const S &y() const { return data()[1]; }
	const S &z() const { return data()[2]; }
	const S &w() const { return data()[3]; }

	// constants
	static Dense Constant(S s) { Dense d; d.setConstant(s); return d; }
	static Dense Constant(Index n, S s) { Dense d(n); d.setConstant(s); return d; }
	static Dense Zero() { return Constant(S(0)); }
	static Dense Zero(Index n) { return Constant(n, S(0)); }
	static Dense Zero(Index r, Index c) { Dense d(r, c); return d; }
	static Dense Ones() { return Constant(S(1)); }
	static Dense Ones(Index n) { return Constant(n, S(1)); }
	static Dense Identity() { Dense d; for (Index i = 0; i < std::min<Index>(d.rows(), d.cols()); i++) d(i, i) = S(1); return d; }
	static Dense Unit(Index i) { Dense d; d[i] = S(1); return d; }
	static Dense Unit(Index n, Index i) { Dense d(n); d[i] = S(1); return d; }
	static Dense UnitX() { return Unit(0); }
	static Dense UnitY() { return Unit(1); }
	static Dense UnitZ() { return Unit(2); }
	static Dense UnitW() { return Unit(3); }
	Dense &setConstant(S s) { for (Index i = 0; i < size(); i++) (*this)[i] = s; return *this; }
	Dense &setZero() { return setConstant(S(0)); }
	Dense &setZero(Index n) { resize(n); return setZero(); }
	Dense &setOnes() { return setConstant(S(1)); }
	Dense &fill(S s) { return setConstant(s); }

	// views and conversions (copies: the reference only reads them)
	DenseOf<S, R, C, true> array() const { DenseOf<S, R, C, true> a; a.st = st; return a; }
	DenseOf<S, R, C, false> matrix() const { DenseOf<S, R, C, false> m; m.st = st; return m; }
	Dense eval() const { return *this; }
	template <typename T> DenseOf<T, R, C, IsArray> cast() const {
		DenseOf<T, R, C, IsArray> o;
		if constexpr (!IsFixed) o.resize(rows(), cols());
		for (Index i = 0; i < size(); i++) o[i] = T((*this)[i]);
		return o;
	}
	DenseOf<S, C, R, IsArray> transpose() const {
		DenseOf<S, C, R, IsArray> t;
		if constexpr (!IsFixed) t.resize(cols(), rows());
		for (Index r = 0; r < rows(); r++)
			for (Index c = 0; c < cols(); c++) t(c, r) = (*this)(r, c);
		return t;
	}
	LineRef<DenseOf<S, R, 1, IsArray>> col(Index j) { return {data() + j * R, 1}; }
	DenseOf<S, R, 1, IsArray> col(Index j) const { DenseOf<S, R, 1, IsArray> v; for (Index i = 0; i < R; i++) v[i] = (*this)(i, j); return v; }
	LineRef<DenseOf<S, 1, C, IsArray>> row(Index i) { return {data() + i, R}; }
	DenseOf<S, 1, C, IsArray> row(Index i) const { DenseOf<S, 1, C, IsArray> v; for (Index j = 0; j < C; j++) v[j] = (*this)(i, j); return v; }

	// reductions, in index order
	S sum() const { S s = S(0); for (Index i = 0; i < size(); i++) s += (*this)[i]; return s; }
	S prod() const { S s = S(1); for (Index i = 0; i < size(); i++) s *= (*this)[i]; return s; }
	S mean() const { return sum() / S(size()); }
	S maxCoeff() const { S m = (*this)[0]; for (Index i = 1; i < size(); i++) m = std::max(m, (*this)[i]); return m; }
	S minCoeff() const { S m = (*this)[0]; for (Index i = 1; i < size(); i++) m = std::min(m, (*this)[i]); return m; }
	template <typename I> S maxCoeff(I *at) const { Index k = 0; for (Index i = 1; i < size(); i++) if ((*this)[i] > (*this)[k]) k = i; *at = I(k); return (*this)[k]; }
	template <typename I> S minCoeff(I *at) const { Index k = 0; for (Index i = 1; i < size(); i++) if ((*this)[i] < (*this)[k]) k = i; *at = I(k); return (*this)[k]; }
	bool all() const { for (Index i = 0; i < size(); i++) if (!(*this)[i]) return false; return true; }
	bool any() const { for (Index i = 0; i < size(); i++) if ((*this)[i]) return true; return false; }
	Index count() const { Index n = 0; for (Index i = 0; i < size(); i++) n += (*this)[i] ? 1 : 0; return n; }
	DenseOf<bool, R, C, true> isFinite() const { DenseOf<bool, R, C, true> m; if constexpr (!IsFixed) m.resize(rows(), cols()); for (Index i = 0; i < size(); i++) m[i] = std::isfinite(double((*this)[i])); return m; }
	bool hasNaN() const { for (Index i = 0; i < size(); i++) if (std::isnan(double((*this)[i]))) return true; return false; }
	bool allFinite() const { for (Index i = 0; i < size(); i++) if (!std::isfinite(double((*this)[i]))) return false; return true; }
	S squaredNorm() const { S s = S(0); for (Index i = 0; i < size(); i++) s += (*this)[i] * (*this)[i]; return s; }
	S norm() const { return std::sqrt(squaredNorm()); }
	template <int P> S lpNorm() const { static_assert(P == Infinity); return cwiseAbs().maxCoeff(); }
	S trace() const { S s = S(0); for (Index i = 0; i < std::min(rows(), cols()); i++) s += (*this)(i, i); return s; }
	Dense normalized() const { const S n = squaredNorm(); if (n > S(0)) return *this / std::sqrt(n); return *this; }
	void normalize() { *this = normalized(); }
	S dot(const Dense &o) const { S s = S(0); for (Index i = 0; i < size(); i++) s += (*this)[i] * o[i]; return s; }
	Dense cross(const Dense &o) const {
		static_assert(SizeAtCompileTime == 3);
		const Dense &a = *this;
		return Dense(a[1] * o[2] - a[2] * o[1], a[2] * o[0] - a[0] * o[2], a[0] * o[1] - a[1] * o[0]);
	}

	// element-wise operations
	template <typename F> Dense map(F f) const { Dense o = *this; for (Index i = 0; i < size(); i++) o[i] = f((*this)[i]); return o; }
	template <typename F> Dense zip(const Dense &b, F f) const { Dense o = *this; for (Index i = 0; i < size(); i++) o[i] = f((*this)[i], b[i]); return o; }
	Dense cwiseMin(const Dense &b) const { return zip(b, [](S p, S q) { return std::min(p, q); }); }
	Dense cwiseMax(const Dense &b) const { return zip(b, [](S p, S q) { return std::max(p, q); }); }
	Dense cwiseMin(S s) const { return map([s](S p) { return std::min(p, s); }); }
	Dense cwiseMax(S s) const { return map([s](S p) { return std::max(p, s); }); }
	Dense cwiseAbs() const { return map([](S p) { return S(std::abs(p)); }); }
	Dense cwiseAbs2() const { return map([](S p) { return p * p; }); }
	Dense cwiseSqrt() const { return map([](S p) { return S(std::sqrt(p)); }); }
	Dense cwiseSign() const { return map([](S p) { return shim::sgn(p); }); }
	Dense cwiseInverse() const { return map([](S p) { return S(1) / p; }); }
	Dense cwiseProduct(const Dense &b) const { return zip(b, [](S p, S q) { return p * q; }); }
	Dense cwiseQuotient(const Dense &b) const { return zip(b, [](S p, S q) { return p / q; }); }
	Dense abs() const { return cwiseAbs(); }
	Dense abs2() const { return cwiseAbs2(); }
	Dense square() const { return cwiseAbs2(); }
	Dense cube() const { return map([](S p) { return p * p * p; }); }
	Dense sqrt() const { return cwiseSqrt(); }
	Dense sign() const { return cwiseSign(); }
	Dense inverse() const requires IsArray { return cwiseInverse(); }
	Dense floor() const { return map([](S p) { return S(std::floor(p)); }); }
	Dense ceil() const { return map([](S p) { return S(std::ceil(p)); }); }
	Dense round() const { return map([](S p) { return S(std::round(p)); }); }
	Dense exp() const { return map([](S p) { return S(std::exp(p)); }); }
	Dense log() const { return map([](S p) { return S(std::log(p)); }); }
	Dense min(const Dense &b) const { return cwiseMin(b); }
	Dense max(const Dense &b) const { return cwiseMax(b); }
	Dense min(S s) const { return cwiseMin(s); }
	Dense max(S s) const { return cwiseMax(s); }

	// small dense matrix algebra
	S determinant() const requires (!IsArray && R == C && R > 0) {
		const Dense &m = *this;
		if constexpr (R == 1) return m(0, 0);
		else if constexpr (R == 2) return m(0, 0) * m(1, 1) - m(0, 1) * m(1, 0);
		else {
			static_assert(R == 3);
			return m(0, 0) * (m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1)) - m(0, 1) * (m(1, 0) * m(2, 2) - m(1, 2) * m(2, 0)) +
			       m(0, 2) * (m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0));
		}
	}
	Dense inverse() const requires (!IsArray && R == C && R > 0) {
		const Dense &m = *this;
		Dense o;
		const S det = determinant();
		if constexpr (R == 1) o(0, 0) = S(1) / m(0, 0);
		else if constexpr (R == 2) {
			o(0, 0) = m(1, 1) / det; o(0, 1) = -m(0, 1) / det;
			o(1, 0) = -m(1, 0) / det; o(1, 1) = m(0, 0) / det;
		} else {
			for (int r = 0; r < 3; r++)
				for (int c = 0; c < 3; c++) {
					const int r1 = (c + 1) % 3, r2 = (c + 2) % 3, c1 = (r + 1) % 3, c2 = (r + 2) % 3;
					o(r, c) = (m(r1, c1) * m(r2, c2) - m(r1, c2) * m(r2, c1)) / det;
				}
		}
		return o;
	}

	// compound assignment
	Dense &operator+=(const Dense &b) { for (Index i = 0; i < size(); i++) (*this)[i] += b[i]; return *this; }
	Dense &operator-=(const Dense &b) { for (Index i = 0; i < size(); i++) (*this)[i] -= b[i]; return *this; }
	Dense &operator*=(S s) { for (Index i = 0; i < size(); i++) (*this)[i] *= s; return *this; }
	Dense &operator/=(S s) { for (Index i = 0; i < size(); i++) (*this)[i] /= s; return *this; }
	Dense &operator*=(const Dense &b) requires IsArray { for (Index i = 0; i < size(); i++) (*this)[i] *= b[i]; return *this; }
	Dense &operator/=(const Dense &b) requires IsArray { for (Index i = 0; i < size(); i++) (*this)[i] /= b[i]; return *this; }
	Dense &operator+=(S s) requires IsArray { for (Index i = 0; i < size(); i++) (*this)[i] += s; return *this; }
	Dense &operator-=(S s) requires IsArray { for (Index i = 0; i < size(); i++) (*this)[i] -= s; return *this; }

	// arithmetic (hidden friends, so that views convert implicitly)
	friend Dense operator+(const Dense &a, const Dense &b) { Dense o = a; o += b; return o; }
	friend Dense operator-(const Dense &a, const Dense &b) { Dense o = a; o -= b; return o; }
	friend Dense operator-(const Dense &a) { return a.map([](S p) { return -p; }); }
	friend Dense operator*(const Dense &a, S s) { Dense o = a; o *= s; return o; }
	friend Dense operator*(S s, const Dense &a) { return a.map([s](S p) { return s * p; }); }
	friend Dense operator/(const Dense &a, S s) { Dense o = a; o /= s; return o; }
	friend Dense operator*(const Dense &a, const Dense &b) requires IsArray { Dense o = a; o *= b; return o; }
	friend Dense operator/(const Dense &a, const Dense &b) requires IsArray { Dense o = a; o /= b; return o; }
	friend Dense operator+(const Dense &a, S s) requires IsArray { Dense o = a; o += s; return o; }
	friend Dense operator+(S s, const Dense &a) requires IsArray { return a.map([s](S p) { return s + p; }); }
	friend Dense operator-(const Dense &a, S s) requires IsArray { Dense o = a; o -= s; return o; }
	friend Dense operator-(S s, const Dense &a) requires IsArray { return a.map([s](S p) { return s - p; }); }
	friend Dense operator/(S s, const Dense &a) requires IsArray { return a.map([s](S p) { return s / p; }); }
	// matrix product
	template <int C2>
	friend DenseOf<S, R, C2, false> operator*(const Dense &a, const DenseOf<S, C, C2, false> &b) requires (!IsArray && !(R == 1 && C == 1 && C2 == 1)) {
		DenseOf<S, R, C2, false> o;
		if constexpr (R == Dynamic || C2 == Dynamic) o.resize(a.rows(), b.cols());
		for (Index r = 0; r < a.rows(); r++)
			for (Index c = 0; c < b.cols(); c++) {
				S s = S(0);
				for (Index k = 0; k < a.cols(); k++) s += a(r, k) * b(k, c);
				o(r, c) = s;
			}
		return o;
	}
	// comparisons: matrices as wholes, arrays element by element
	friend bool operator==(const Dense &a, const Dense &b) requires (!IsArray) { for (Index i = 0; i < a.size(); i++) if (a[i] != b[i]) return false; return true; }
	friend bool operator!=(const Dense &a, const Dense &b) requires (!IsArray) { return !(a == b); }
	using Mask = DenseOf<bool, R, C, true>;
	template <typename F> Mask test(const Dense &b, F f) const { Mask m; if constexpr (!IsFixed) m.resize(rows(), cols()); for (Index i = 0; i < size(); i++) m[i] = f((*this)[i], b[i]); return m; }
	template <typename F> Mask test(S s, F f) const { Mask m; if constexpr (!IsFixed) m.resize(rows(), cols()); for (Index i = 0; i < size(); i++) m[i] = f((*this)[i], s); return m; }
	friend Mask operator<(const Dense &a, const Dense &b) requires IsArray { return a.test(b, [](S p, S q) { return p < q; }); }
	friend Mask operator<=(const Dense &a, const Dense &b) requires IsArray { return a.test(b, [](S p, S q) { return p <= q; }); }
	friend Mask operator>(const Dense &a, const Dense &b) requires IsArray { return a.test(b, [](S p, S q) { return p > q; }); }
	friend Mask operator>=(const Dense &a, const Dense &b) requires IsArray { return a.test(b, [](S p, S q) { return p >= q; }); }
	friend Mask operator==(const Dense &a, const Dense &b) requires IsArray { return a.test(b, [](S p, S q) { return p == q; }); }
	friend Mask operator!=(const Dense &a, const Dense &b) requires IsArray { return a.test(b, [](S p, S q) { return p != q; }); }
	friend Mask operator<(const Dense &a, S s) requires IsArray { return a.test(s, [](S p, S q) { return p < q; }); }
	friend Mask operator<=(const Dense &a, S s) requires IsArray { return a.test(s, [](S p, S q) { return p <= q; }); }
	friend Mask operator>(const Dense &a, S s) requires IsArray { return a.test(s, [](S p, S q) { return p > q; }); }
	friend Mask operator>=(const Dense &a, S s) requires IsArray { return a.test(s, [](S p, S q) { return p >= q; }); }
	friend Mask operator==(const Dense &a, S s) requires IsArray { return a.test(s, [](S p, S q) { return p == q; }); }
	friend Mask operator!=(const Dense &a, S s) requires IsArray { return a.test(s, [](S p, S q) { return p != q; }); }
	friend Dense operator&&(const Dense &a, const Dense &b) requires (IsArray && std::is_same_v<S, bool>) { return a.zip(b, [](S p, S q) { return p && q; }); }
	friend Dense operator||(const Dense &a, const Dense &b) requires (IsArray && std::is_same_v<S, bool>) { return a.zip(b, [](S p, S q) { return p || q; }); }
	friend Dense operator!(const Dense &a) requires (IsArray && std::is_same_v<S, bool>) { return a.map([](S p) { return !p; }); }

	// printing
	struct WithFormat { const Dense &d; IOFormat f; };
	WithFormat format(const IOFormat &f) const { return {*this, f}; }
	friend std::ostream &operator<<(std::ostream &os, const Dense &d) {
		for (Index r = 0; r < d.rows(); r++) {
			for (Index c = 0; c < d.cols(); c++) os << (c ? " " : "") << d(r, c);
			if (r + 1 < d.rows()) os << "\n";
		}
		return os;
	}
	friend std::ostream &operator<<(std::ostream &os, const WithFormat &w) {
		const auto p = os.precision();
		if (w.f.precision >= 0) os.precision(w.f.precision);
		for (Index i = 0; i < w.d.size(); i++) os << (i ? " " : "") << w.d[i];
		os.precision(p);
		return os;
	}
};

#define GARM_SHIM_TYPES(S, s)                               \
	using Vector2##s = Matrix<S, 2, 1>;                     \
	using Vector3##s = Matrix<S, 3, 1>;                     \
	using Vector4##s = Matrix<S, 4, 1>;                     \
	using VectorX##s = Matrix<S, Dynamic, 1>;               \
	using RowVector2##s = Matrix<S, 1, 2>;                  \
	using RowVector3##s = Matrix<S, 1, 3>;                  \
	using Matrix2##s = Matrix<S, 2, 2>;                     \
	using Matrix3##s = Matrix<S, 3, 3>;                     \
	using Matrix4##s = Matrix<S, 4, 4>;                     \
	using MatrixX##s = Matrix<S, Dynamic, Dynamic>;         \
	using Array2##s = Array<S, 2, 1>;                       \
	using Array3##s = Array<S, 3, 1>;                       \
	using Array4##s = Array<S, 4, 1>;                       \
	using ArrayX##s = Array<S, Dynamic, 1>;
GARM_SHIM_TYPES(double, d)
GARM_SHIM_TYPES(float, f)
GARM_SHIM_TYPES(int, i)
#undef GARM_SHIM_TYPES

// Map and Ref over a plain double vector: a pointer and a length that read and write in place.
template <typename V, int Opt = Unaligned> class Map {
public:
	using Plain = std::remove_const_t<V>;
	using Scalar = typename Plain::Scalar;
	using Ptr = std::conditional_t<std::is_const_v<V>, const Scalar *, Scalar *>;
	Map(Ptr p, Index n) : _p(p), _n(n) { }
	Index size() const { return _n; }
	Index rows() const { return _n; }
	Ptr data() const { return _p; }
	Scalar &operator[](Index i) const requires (!std::is_const_v<V>) { return _p[i]; }
	Scalar operator[](Index i) const requires std::is_const_v<V> { return _p[i]; }
	Plain eval() const { Plain v(_n); for (Index i = 0; i < _n; i++) v[i] = _p[i]; return v; }
	operator Plain() const { return eval(); }
	Map &operator=(const Plain &o) requires (!std::is_const_v<V>) { assert(o.size() == _n); for (Index i = 0; i < _n; i++) _p[i] = o[i]; return *this; }
	Scalar squaredNorm() const { return eval().squaredNorm(); }
	Scalar norm() const { return eval().norm(); }
	Scalar dot(const Plain &o) const { return eval().dot(o); }
private:
	Ptr _p;
	Index _n;
};

template <typename V, int Opt = Unaligned> class Ref : public Map<V, Opt> {
public:
	using Base = Map<V, Opt>;
	using Plain = typename Base::Plain;
	Ref(std::conditional_t<std::is_const_v<V>, const Plain &, Plain &> v) : Base(v.data(), v.size()) { }
	template <int O2> Ref(const Map<V, O2> &m) : Base(m.data(), m.size()) { }
	template <int O2> Ref(const Map<std::remove_const_t<V>, O2> &m) requires std::is_const_v<V> : Base(m.data(), m.size()) { }
	using Base::operator=;
};

}  // namespace Eigen
