// Test-infrastructure shim: dense ROOT TMatrixT / TVectorT with the members
// the reference's likelihood uses (zero-initialised (rows, cols)
// construction, m[i][j], the kInverted constructor, EigenVectors of a
// symmetric matrix with eigenvalues in descending order, column views).  The
// inverse (Gauss-Jordan with partial pivoting) and the eigen decomposition
// (cyclic Jacobi) are this shim's own linear algebra, not ROOT's: results
// that pass through them agree with ROOT's to rounding only.
#ifndef RPWA_SHIM_TMATRIXT_H
#define RPWA_SHIM_TMATRIXT_H

#include <algorithm>
#include <cmath>
#include <numeric>
#include <stdexcept>
#include <vector>

#include "RtypesShim.h"

template<typename T> class TMatrixT;

template<typename T>
class TMatrixTColumn_const {
public:
	TMatrixTColumn_const(const TMatrixT<T>& m, int col) : _m(&m), _col(col) {}
	const TMatrixT<T>* matrix() const { return _m; }
	int                column() const { return _col; }
private:
	const TMatrixT<T>* _m;
	int                _col;
};

template<typename T>
class TVectorT {
public:
	TVectorT() {}
	explicit TVectorT(int n) : _v(n, T(0)) {}
	TVectorT(const TMatrixTColumn_const<T>& c);
	T&       operator[](int i)       { return _v[i]; }
	const T& operator[](int i) const { return _v[i]; }
	T&       operator()(int i)       { return _v[i]; }
	const T& operator()(int i) const { return _v[i]; }
	int      GetNrows() const        { return (int)_v.size(); }
	void     ResizeTo(int n)         { _v.resize(n, T(0)); }
private:
	std::vector<T> _v;
};

template<typename T>
class TMatrixT {
public:
	enum EMatrixCreatorsOp1 { kZero, kUnit, kTransposed, kInverted, kAtA };

	TMatrixT() {}
	TMatrixT(int nRows, int nCols) : _r(nRows), _c(nCols), _d((size_t)nRows * nCols, T(0)) {}
	TMatrixT(EMatrixCreatorsOp1 op, const TMatrixT& m)
	{
		if (op != kInverted)
			throw std::logic_error("TMatrixT shim: only kInverted is provided");
		*this = m.inverse();
	}

	T*       operator[](int i)              { return &_d[(size_t)i * _c]; }
	const T* operator[](int i) const        { return &_d[(size_t)i * _c]; }
	T&       operator()(int i, int j)       { return _d[(size_t)i * _c + j]; }
	const T& operator()(int i, int j) const { return _d[(size_t)i * _c + j]; }
	int      GetNrows() const               { return _r; }
	int      GetNcols() const               { return _c; }

	// eigenvectors (columns) and eigenvalues of a symmetric matrix, eigenvalues descending
	TMatrixT EigenVectors(TVectorT<T>& eigenValues) const
	{
		const int n = _r;
		TMatrixT  a(*this), v(n, n);
		for (int i = 0; i < n; ++i)
			v(i, i) = 1;
		for (int sweep = 0; sweep < 100; ++sweep) {
			T off = 0, tot = 0;
			for (int i = 0; i < n; ++i)
				for (int j = 0; j < n; ++j) {
					tot += a(i, j) * a(i, j);
					if (i != j)
						off += a(i, j) * a(i, j);
				}
			if (off <= 1e-30 * tot)
				break;
			for (int p = 0; p < n; ++p)
				for (int q = p + 1; q < n; ++q) {
					if (a(p, q) == 0)
						continue;
					const T theta = (a(q, q) - a(p, p)) / (2 * a(p, q));
					const T t     = (theta >= 0 ? 1 : -1) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
					const T c     = 1 / std::sqrt(t * t + 1), s = t * c;
					for (int k = 0; k < n; ++k) {
						const T akp = a(k, p), akq = a(k, q);
						a(k, p) = c * akp - s * akq;
						a(k, q) = s * akp + c * akq;
					}
					for (int k = 0; k < n; ++k) {
						const T apk = a(p, k), aqk = a(q, k);
						a(p, k) = c * apk - s * aqk;
						a(q, k) = s * apk + c * aqk;
					}
					for (int k = 0; k < n; ++k) {
						const T vkp = v(k, p), vkq = v(k, q);
						v(k, p) = c * vkp - s * vkq;
						v(k, q) = s * vkp + c * vkq;
					}
				}
		}
		std::vector<int> order(n);
		std::iota(order.begin(), order.end(), 0);
		std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return a(x, x) > a(y, y); });
		eigenValues = TVectorT<T>(n);
		TMatrixT vs(n, n);
		for (int k = 0; k < n; ++k) {
			eigenValues[k] = a(order[k], order[k]);
			for (int i = 0; i < n; ++i)
				vs(i, k) = v(i, order[k]);
		}
		return vs;
	}

private:

	TMatrixT inverse() const
	{
		const int n = _r;
		if (n != _c)
			throw std::logic_error("TMatrixT shim: inverse of a non-square matrix");
		TMatrixT a(*this), b(n, n);
		for (int i = 0; i < n; ++i)
			b(i, i) = 1;
		for (int col = 0; col < n; ++col) {
			int piv = col;
			for (int i = col + 1; i < n; ++i)
				if (std::fabs(a(i, col)) > std::fabs(a(piv, col)))
					piv = i;
			if (a(piv, col) == 0)
				throw std::runtime_error("TMatrixT shim: singular matrix");
			for (int k = 0; k < n; ++k) {
				std::swap(a(col, k), a(piv, k));
				std::swap(b(col, k), b(piv, k));
			}
			const T d = a(col, col);
			for (int k = 0; k < n; ++k) {
				a(col, k) /= d;
				b(col, k) /= d;
			}
			for (int i = 0; i < n; ++i) {
				if (i == col || a(i, col) == 0)
					continue;
				const T f = a(i, col);
				for (int k = 0; k < n; ++k) {
					a(i, k) -= f * a(col, k);
					b(i, k) -= f * b(col, k);
				}
			}
		}
		return b;
	}

	int            _r = 0, _c = 0;
	std::vector<T> _d;
};

template<typename T>
TVectorT<T>::TVectorT(const TMatrixTColumn_const<T>& c) : _v(c.matrix()->GetNrows())
{
	for (int i = 0; i < (int)_v.size(); ++i)
		_v[i] = (*c.matrix())(i, c.column());
}

#endif
