// gram_tc.cu -- tensor-core (tcgen05) Gram kernel for the integral matrices.
#include "pwa_internal.h"

namespace pwa {

int launchGramTc(const GramArgs&, int, int, cudaStream_t, double*, double*, size_t)
{
	return setError(kErrUnsupported, "tensor-core Gram kernel not available in this build");
}

}  // namespace pwa
