/* KEncode instantiation for batches that mix presets: each texture's
   kDenoise read at run time, draft and refinement passes; outlined shape. */
#define NEBC7_PASS __noinline__
#define NEBC7_ONCE __noinline__
#include "bc7_encode_entry.cuh"

NEBC7_INSTANTIATE_ENCODE(nebc7::kAnyDenoise, true, nebc7::kShapeOutlined)
