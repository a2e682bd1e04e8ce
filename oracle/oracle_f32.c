/* Single-precision oracle (the reference's realkind = sp build). Test infrastructure only. */
#define REAL float
#define ORC(name) orc_f32_##name
#include "axisem_oracle.c"
