// Test-infrastructure shim: see TMatrixT.h.
#include "TMatrixT.h"
