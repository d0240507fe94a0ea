// Stand-in for RAPTor's phong_shader.h (test infrastructure): see raptor_stand_in.h.
#pragma once
#include "raptor_stand_in.h"
