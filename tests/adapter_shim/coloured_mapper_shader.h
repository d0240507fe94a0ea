// Stand-in for RAPTor's coloured_mapper_shader.h (test infrastructure): see raptor_stand_in.h.
#pragma once
#include "raptor_stand_in.h"
