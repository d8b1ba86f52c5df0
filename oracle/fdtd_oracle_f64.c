/* Double-precision instance of the CPU oracle (test infrastructure only). */
#define REAL double
#define SFX(name) name##_f64
#include "fdtd_oracle_impl.h"
