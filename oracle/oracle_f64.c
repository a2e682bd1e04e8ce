/* Double-precision oracle (the reference's realkind = dp build). Test infrastructure only. */
#define REAL double
#define ORC(name) orc_f64_##name
#include "axisem_oracle.c"
