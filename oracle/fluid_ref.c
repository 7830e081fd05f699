/* C restatement of the tinyfluids time step -- TEST INFRASTRUCTURE ONLY.
 *
 * The same scheme as oracle/fluid_np.py (which cites the reference
 * file:line for every op), written in C so that larger parity cases and the
 * timed CPU baseline run in seconds.  Built by oracle/build.py with
 * -O2 -ffp-contract=off -fno-fast-math -fopenmp; no target-specific flags,
 * so x86-64 and aarch64 builds give the same bits.  The float entry points
 * (suffix _f32) are bit-identical to fluid_np.py at float32; the double entry
 * points (_f64) are the FP64 oracle.
 */
#include <math.h>
#include <stdlib.h>

#define R float
#define SQRT sqrtf
#define FN(x) x##_f32
#include "fluid_ref_impl.h"
#undef R
#undef SQRT
#undef FN

#define R double
#define SQRT sqrt
#define FN(x) x##_f64
#include "fluid_ref_impl.h"
#undef R
#undef SQRT
#undef FN

#ifdef _OPENMP
#include <omp.h>
int orc_max_threads(void) { return omp_get_max_threads(); }
void orc_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }
#else
int orc_max_threads(void) { return 1; }
void orc_set_threads(int n) { (void)n; }
#endif
