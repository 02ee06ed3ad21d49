/* KEncode instantiation: differences halved (kDenoise 1), draft passes only; compact shape. */
#define NEBC7_SHARED
#include "bc7_encode_entry.cuh"

NEBC7_INSTANTIATE_ENCODE(1, false, nebc7::kShapeCompact)
