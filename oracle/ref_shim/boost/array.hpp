// Test-infrastructure shim: boost::array as std::array (aggregate, same
// brace initialisation).  Only used to compile the reference's own sources
// into the checker library under oracle/_ref.
#ifndef RPWA_SHIM_ARRAY_HPP
#define RPWA_SHIM_ARRAY_HPP
#include <array>
namespace boost {
	template<typename T, std::size_t N>
	using array = std::array<T, N>;
}
#endif
