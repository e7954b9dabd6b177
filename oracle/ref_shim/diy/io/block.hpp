// Single-process DIY stand-in (test oracle only); all declarations live in types.hpp.
#pragma once
#include "../types.hpp"
