// ipp_m7.h stand-in for the executed-reference checker (the reference
// includes it beside ipp.h; the two functions used live in ipp.h).
#pragma once
#include "ipp.h"
