// lbmx compat: cuda-lbm scenarios include the functor collection
// (src/functors/includes.cuh) for the BC_flag names; the boundary functors
// themselves run inside the engine, selected by those flags.
#ifndef FUNCTOR_INCLUDES_H
#define FUNCTOR_INCLUDES_H
#include "core/lbm_constants.cuh"
#endif
