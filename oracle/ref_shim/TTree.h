// Test-infrastructure shim: an in-memory TTree over borrowed columns.  An
// amplitude tree holds, per entry, nSubAmps complex<double> values (one
// amplitudeTreeLeaf branch named "amplitude"); an event tree holds named
// double columns (the on-the-fly binning variables).  GetEntry(i) fills the
// addresses given to SetBranchAddress, as ROOT does.
#ifndef RPWA_SHIM_TTREE_H
#define RPWA_SHIM_TTREE_H
#include <complex>
#include <map>
#include <string>
#include <vector>
#include "amplitudeTreeLeaf.h"
class TTree {
public:
	explicit TTree(long nEntries) : _n(nEntries) {}
	void setAmplitudes(const std::complex<double>* amps, unsigned int nSubAmps)
	{
		_amps    = amps;
		_nSubAmp = nSubAmps;
	}
	void addColumn(const std::string& name, const double* values) { _cols[name] = values; }
	long GetEntries()     const { return _n; }
	long GetEntriesFast() const { return _n; }
	int SetBranchAddress(const char* name, rpwa::amplitudeTreeLeaf** leaf)
	{
		if (!_amps || std::string(name) != "amplitude")
			return -5;
		if (!*leaf)
			*leaf = &_leaf;
		_leafAddr = leaf;
		return 0;
	}
	int SetBranchAddress(const char* name, double* addr)
	{
		if (!_cols.count(name))
			return -5;
		_colAddr[name] = addr;
		return 0;
	}
	int GetEntry(long i)
	{
		if (i < 0 || i >= _n)
			return 0;
		if (_leafAddr) {
			rpwa::amplitudeTreeLeaf* l = *_leafAddr;
			l->_subAmps.assign(_amps + (size_t)i * _nSubAmp, _amps + (size_t)(i + 1) * _nSubAmp);
		}
		for (auto& c : _colAddr)
			*c.second = _cols[c.first][i];
		return 1;
	}
private:
	long                                  _n;
	const std::complex<double>*           _amps     = nullptr;
	unsigned int                          _nSubAmp  = 0;
	rpwa::amplitudeTreeLeaf               _leaf;
	rpwa::amplitudeTreeLeaf**             _leafAddr = nullptr;
	std::map<std::string, const double*>  _cols;
	std::map<std::string, double*>        _colAddr;
};
#endif
