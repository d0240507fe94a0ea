// Stand-in for RAPTor's light.h (test infrastructure): see raptor_stand_in.h.
#pragma once
#include "raptor_stand_in.h"
