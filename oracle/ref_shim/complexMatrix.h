// Test-infrastructure shim: the element access of rpwa::complexMatrix that
// pwaLikelihood::getIntegralMatrices uses.
#ifndef RPWA_SHIM_COMPLEXMATRIX_H
#define RPWA_SHIM_COMPLEXMATRIX_H
#include <complex>
#include <vector>
#include "TObject.h"
namespace rpwa {
	class complexMatrix : public TObject {
	public:
		complexMatrix() {}
		complexMatrix(const int i, const int j) { resizeTo(i, j); }
		void resizeTo(const int i, const int j) { _r = i; _c = j; _m.assign((size_t)i * j, 0); }
		void set(const int i, const int j, const std::complex<double>& c) { _m[(size_t)i * _c + j] = c; }
		std::complex<double> get(const int i, const int j) const { return _m[(size_t)i * _c + j]; }
		std::complex<double> operator()(const int i, const int j) const { return get(i, j); }
		unsigned int nRows() const { return _r; }
		unsigned int nCols() const { return _c; }
	private:
		int                                _r = 0, _c = 0;
		std::vector<std::complex<double> > _m;
	};
}
#endif
