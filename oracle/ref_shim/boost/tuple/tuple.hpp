// Test-infrastructure shim: boost::tuples mapped onto std::tuple (the
// reference uses tuple, make_tuple and get<i> only).  Only used to compile
// the reference's own sources into the checker library under oracle/_ref.
#ifndef RPWA_SHIM_TUPLE_HPP
#define RPWA_SHIM_TUPLE_HPP
#include <tuple>
namespace boost {
	namespace tuples {
		using std::tuple;
		using std::make_tuple;
		using std::get;
	}
	using tuples::tuple;
	using std::get;
}
#endif
