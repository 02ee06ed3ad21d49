/* Staged encode kernels: differences halved (kDenoise 1: /slow and /data);
   one kernel per pass, the pass-level routines out of line. */
#define NEBC7_PASS __noinline__
#define NEBC7_ONCE __noinline__
#include "bc7_staged_entry.cuh"

NEBC7_INSTANTIATE_STAGED(1)
