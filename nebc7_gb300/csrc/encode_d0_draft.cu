/* KEncode instantiation: exact differences (kDenoise 0), draft passes only; compact shape. */
#define NEBC7_SHARED
/* the fast passes and the final pack out of line, each with its own register
   allocation: 1074 -> 1150 Mpx/s on a 1024x1024 photo */
#define NEBC7_ONCE __noinline__
#include "bc7_encode_entry.cuh"

NEBC7_INSTANTIATE_ENCODE(0, false, nebc7::kShapeCompact)
