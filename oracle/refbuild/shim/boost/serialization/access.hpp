// Declaration-only stand-in for Boost.Serialization (never executed).
#pragma once
namespace boost { namespace serialization {
class access {};
template <class T> inline T &make_nvp(const char *, T &t) { return t; }
} }
#define BOOST_SERIALIZATION_NVP(x) (x)
