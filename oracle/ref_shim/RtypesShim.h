// Test-infrastructure shim: the ROOT basic types and class macros that the
// reference's likelihood and integral sources name.  No ROOT I/O: the
// streamer hooks exist only so that the reference's sources compile.  Only
// used to compile the reference's own sources into the checker library under
// oracle/_ref.
#ifndef RPWA_SHIM_RTYPES_H
#define RPWA_SHIM_RTYPES_H
#include <cstdlib>
typedef char      Option_t;
typedef bool      Bool_t;
typedef int       Int_t;
typedef long long Long64_t;
typedef double    Double_t;
static const bool kTRUE  = true;
static const bool kFALSE = false;
class TClass;
class TBuffer;
#define ClassDef(name, id)                                   \
	public:                                                  \
	static TClass* Class() { return nullptr; }               \
	virtual void   Streamer(TBuffer&);
#define ClassImp(name)
#endif
