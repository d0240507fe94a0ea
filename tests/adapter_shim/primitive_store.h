// Stand-in for RAPTor's primitive_store.h (test infrastructure): see raptor_stand_in.h.
#pragma once
#include "raptor_stand_in.h"
