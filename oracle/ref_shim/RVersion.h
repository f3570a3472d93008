// Test-infrastructure shim (see RtypesShim.h).
#ifndef RPWA_SHIM_RVERSION_H
#define RPWA_SHIM_RVERSION_H
#define ROOT_VERSION(a, b, c) (((a) << 16) + ((b) << 8) + (c))
#define ROOT_VERSION_CODE ROOT_VERSION(6, 20, 0)
#endif
