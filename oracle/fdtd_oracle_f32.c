/* Single-precision instance of the CPU oracle (test infrastructure only). */
#define REAL float
#define SFX(name) name##_f32
#define GPO_PRIMARY 1
#include "fdtd_oracle_impl.h"
