// Test-infrastructure shim: wall-clock stopwatch with ROOT's TStopwatch
// interface (Start, Stop, RealTime, CpuTime).
#ifndef RPWA_SHIM_TSTOPWATCH_H
#define RPWA_SHIM_TSTOPWATCH_H
#include <chrono>
#include "RtypesShim.h"
class TStopwatch {
public:
	TStopwatch() { Start(); }
	void Start(bool reset = true)
	{
		if (reset)
			_total = 0;
		_t0      = std::chrono::steady_clock::now();
		_running = true;
	}
	void Stop()
	{
		if (_running)
			_total += std::chrono::duration<double>(std::chrono::steady_clock::now() - _t0).count();
		_running = false;
	}
	double RealTime() { Stop(); return _total; }
	double CpuTime()  { return RealTime(); }
private:
	std::chrono::steady_clock::time_point _t0;
	double                                _total   = 0;
	bool                                  _running = false;
};
#endif
