// Declaration-only stand-in for Boost.StringAlgo (never executed on the traced path).
#pragma once
#include <string>
namespace boost {
bool iequals(const std::string &, const std::string &);
namespace algorithm { void to_lower(std::string &); void to_upper(std::string &); }
}
