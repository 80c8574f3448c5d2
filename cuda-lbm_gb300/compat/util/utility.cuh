// lbmx compat: src/util/utility.cuh is included for checkCudaErrors; engine
// calls return status codes instead of exiting.
#ifndef UTILITY_H
#define UTILITY_H
#include <cstdio>
#endif
