// Declaration-only stand-in for a Boost archive header (never executed).
#pragma once
#include "boost/serialization/access.hpp"
namespace boost { namespace archive { class text_iarchive {}; } }
