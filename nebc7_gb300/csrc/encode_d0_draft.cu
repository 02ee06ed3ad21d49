/* KEncode instantiation: exact differences (kDenoise 0), draft passes only; compact shape. */
#define NEBC7_SHARED
#include "bc7_encode_entry.cuh"

NEBC7_INSTANTIATE_ENCODE(0, false, nebc7::kShapeCompact)
