// Declaration-only stand-in for Boost.Filesystem (never executed on the traced path).
#pragma once
#include <string>
namespace boost { namespace filesystem {
std::string extension(const std::string &);
} }
