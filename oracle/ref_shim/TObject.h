// Test-infrastructure shim (see RtypesShim.h).
#ifndef RPWA_SHIM_TOBJECT_H
#define RPWA_SHIM_TOBJECT_H
#include "RtypesShim.h"
class TObject {
public:
	virtual ~TObject() {}
};
#endif
