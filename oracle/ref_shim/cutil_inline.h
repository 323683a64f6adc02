// Stand-in for the reference's vendored cutil_inline.h: only cutilSafeCall.
#pragma once
#include "cuda_runtime.h"
#include <cstdio>
#define cutilSafeCall(x) (x)
