// Test-infrastructure shim: the amplitude leaf of one event (its incoherent
// sub-amplitudes), as read through TTree::GetEntry.
#ifndef RPWA_SHIM_AMPLITUDETREELEAF_H
#define RPWA_SHIM_AMPLITUDETREELEAF_H
#include <complex>
#include <vector>
#include "TObject.h"
namespace rpwa {
	class amplitudeTreeLeaf : public TObject {
	public:
		unsigned int                nmbIncohSubAmps() const              { return (unsigned int)_subAmps.size(); }
		const std::complex<double>& incohSubAmp(const unsigned int i) const { return _subAmps[i]; }
		std::vector<std::complex<double> > _subAmps;
	};
}
#endif
