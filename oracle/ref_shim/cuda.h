// Host stand-in for <cuda.h> (TEST INFRASTRUCTURE ONLY): the reference-side
// parity harness needs only what cuda_runtime.h provides.
#pragma once
#include "cuda_runtime.h"
