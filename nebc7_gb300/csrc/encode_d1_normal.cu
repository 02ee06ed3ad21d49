/* KEncode instantiation: differences halved (kDenoise 1), draft and refinement passes with
   the stepped full searches; compact shape (the default preset). */
#define NEBC7_SHARED
/* the reduced tables in the per-x layout (its time is in the Mode6Index2 refinement) */
#define NEBC7_REDUCED_BY_DIFF 0
#include "bc7_encode_entry.cuh"

NEBC7_INSTANTIATE_ENCODE(1, true, nebc7::kShapeCompact)
