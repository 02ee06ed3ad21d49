/* KEncode instantiation for batches that mix presets: each texture's
   kDenoise read at run time, draft and refinement passes; outlined shape. */
#include "bc7_encode_entry.cuh"

NEBC7_INSTANTIATE_ENCODE(nebc7::kAnyDenoise, true, nebc7::kShapeOutlined)
