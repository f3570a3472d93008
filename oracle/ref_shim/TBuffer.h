// Test-infrastructure shim (see RtypesShim.h): ROOT object streaming is not
// available; the checker never reads or writes ROOT files.
#ifndef RPWA_SHIM_TBUFFER_H
#define RPWA_SHIM_TBUFFER_H
#include "RtypesShim.h"
class TBuffer {
public:
	bool IsReading() const { return false; }
	void ReadClassBuffer(TClass*, void*) { std::abort(); }
	void WriteClassBuffer(TClass*, void*) { std::abort(); }
};
#endif
