/*
 * Definitions of the KEncode launchers declared in bc7_encode.cuh; included
 * by the per-instantiation translation units only.
 */
#pragma once

#include "bc7_encode.cuh"

namespace nebc7 {

template<int kD, bool NORMAL>
cudaError_t LaunchEncodeKernel(int grid, cudaStream_t stream, const Job& job, const LevelTables& T, const Params& P)
{
	KEncode<kD, NORMAL><<<grid, kWarpsPerCta * 32, 0, stream>>>(job, T, P);
	return cudaGetLastError();
}

template<int kD, bool NORMAL>
cudaError_t EncodeKernelOccupancy(int* ctasPerSm)
{
	return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctasPerSm, KEncode<kD, NORMAL>, kWarpsPerCta * 32, 0);
}

} // namespace nebc7

#define NEBC7_INSTANTIATE_ENCODE(KD, NORMAL) \
	template cudaError_t nebc7::LaunchEncodeKernel<KD, NORMAL>(int, cudaStream_t, const nebc7::Job&, \
		const nebc7::LevelTables&, const nebc7::Params&); \
	template cudaError_t nebc7::EncodeKernelOccupancy<KD, NORMAL>(int*);
