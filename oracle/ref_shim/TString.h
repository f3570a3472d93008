// Test-infrastructure shim (see RtypesShim.h): only the class name is used.
#ifndef RPWA_SHIM_TSTRING_H
#define RPWA_SHIM_TSTRING_H
#include "RtypesShim.h"
class TString {};
#endif
