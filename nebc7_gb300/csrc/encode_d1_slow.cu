/* KEncode instantiation: differences halved (kDenoise 1), draft, refinement and full-search passes;
   outlined shape (/slow and /data, where the full searches dominate). */
#define NEBC7_PASS __noinline__
#define NEBC7_ONCE __noinline__
#include "bc7_encode_entry.cuh"

NEBC7_INSTANTIATE_ENCODE(1, true, nebc7::kShapeOutlined)
