// Test-infrastructure shim: the Boost version the progress-display header
// switches on.
#ifndef RPWA_SHIM_BOOST_VERSION_HPP
#define RPWA_SHIM_BOOST_VERSION_HPP
#define BOOST_VERSION 107400
#endif
