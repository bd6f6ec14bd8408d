/* Test infrastructure: instantiates the CPU restatement of the reference implicit step,
 * of the COUPLED Jacobian mode, and of the FEM demo's block-sparse CG, in FP32 and FP64
 * (see oc_oracle.h).  Build with -O2 -ffp-contract=off and without
 * -ffast-math so every operation rounds as written. */
#include "oc_oracle.h"

#include <math.h>
#include <stddef.h>
#include <stdlib.h>

#define REAL float
#define SQRT sqrtf
#define SFX(name) name##_f32
#include "oc_oracle_impl.h"
#include "oc_coupled_impl.h"
#include "oc_bsr_impl.h"
#undef REAL
#undef SQRT
#undef SFX

#define REAL double
#define SQRT sqrt
#define SFX(name) name##_f64
#include "oc_oracle_impl.h"
#include "oc_coupled_impl.h"
#include "oc_bsr_impl.h"
#undef REAL
#undef SQRT
#undef SFX
