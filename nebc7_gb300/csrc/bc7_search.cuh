/*
 * BC7 block encoder for sm_103a -- refinement and full searches (the
 * reference's "normal" and "slow" passes).
 */
#pragma once

#include "bc7_fast.cuh"

namespace nebc7 {

/* Set when the library is built with the refinement / full-search passes. */
constexpr bool kHasNormalPasses = false;

template<int kD>
__device__ void NormalPasses(WarpState& st, CellRegs& R, const Params& P, const LevelTables& T, int* status, int lane)
{
	(void)st;
	(void)R;
	(void)P;
	(void)T;
	(void)status;
	(void)lane;
}

} // namespace nebc7
