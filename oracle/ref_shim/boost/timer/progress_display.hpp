// Test-infrastructure shim: a progress display that prints nothing (the
// checker runs inside tests).
#ifndef RPWA_SHIM_PROGRESS_DISPLAY_HPP
#define RPWA_SHIM_PROGRESS_DISPLAY_HPP
#include <ostream>
#include <string>
namespace boost {
	namespace timer {
		class progress_display {
		public:
			progress_display(unsigned long, std::ostream&, const std::string& = "\n",
			                 const std::string& = "", const std::string& = "") {}
			unsigned long operator++() { return ++_count; }
		private:
			unsigned long _count = 0;
		};
	}
}
#endif
