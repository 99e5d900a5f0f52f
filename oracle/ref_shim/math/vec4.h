// vec4.h -- forwards to the scalar stand-in for Embree's vector math (reference build only).
#pragma once
#include "embree_scalar_math.h"
