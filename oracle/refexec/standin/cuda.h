// cuda.h stand-in for the executed-reference checker: the kernel sources
// include it, and everything they use comes from ctref_cuda.h.
#pragma once
#include "ctref_cuda.h"
