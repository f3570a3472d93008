// Test-infrastructure shim: boost::numeric_cast as a range-checked
// static_cast.  Only used to compile the reference's own sources into the
// checker library under oracle/_ref.
#ifndef RPWA_SHIM_NUMERIC_CAST_HPP
#define RPWA_SHIM_NUMERIC_CAST_HPP
#include <limits>
#include <stdexcept>
namespace boost {
	template<typename To, typename From>
	To numeric_cast(From x)
	{
		if (static_cast<From>(static_cast<To>(x)) != x)
			throw std::range_error("numeric_cast: value out of range");
		return static_cast<To>(x);
	}
}
#endif
