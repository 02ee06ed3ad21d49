/* KEncode instantiation: exact differences (kDenoise 0), draft, refinement and full-search passes. */
#include "bc7_encode_entry.cuh"

NEBC7_INSTANTIATE_ENCODE(0, true)
