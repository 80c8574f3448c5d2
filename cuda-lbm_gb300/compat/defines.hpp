// lbmx compat: the configuration macros a cuda-lbm scenario header expects
// (the reference selects them in src/defines.hpp:4-70).  The lattice size
// comes from the including translation unit: define NX and NY first.
#ifndef DEFINES_H
#define DEFINES_H
#define D2Q9
#ifndef NX
#error "lbmx compat: define NX and NY (lattice size) before including a scenario header"
#endif
#ifndef SCALE
#define SCALE 1
#endif
#ifndef NZ
#define NZ 1
#endif
#define BLOCK_SIZE 16
#endif
