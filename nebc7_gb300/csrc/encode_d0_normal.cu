/* KEncode instantiation: exact differences (kDenoise 0), draft, refinement and full-search passes;
   outlined shape (the precise preset runs the full searches on most blocks). */
#define NEBC7_PASS __noinline__
#define NEBC7_ONCE __noinline__
#include "bc7_encode_entry.cuh"

NEBC7_INSTANTIATE_ENCODE(0, true, nebc7::kShapeOutlined)
