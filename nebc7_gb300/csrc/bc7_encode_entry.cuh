/*
 * Definitions of the KEncode launchers declared in bc7_encode.cuh; included
 * by the per-instantiation translation units only.
 */
#pragma once

#include "bc7_encode.cuh"

namespace nebc7 {

/* Lets the kernel use more than the default 48 KB of dynamic shared memory
   (once per process and device; idempotent). */
template<int kD, bool NORMAL, int SHAPE>
cudaError_t PrepareEncodeKernel()
{
	return cudaFuncSetAttribute(KEncode<kD, NORMAL, SHAPE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		int(EncodeSharedBytes<NORMAL>()));
}

template<int kD, bool NORMAL, int SHAPE>
cudaError_t LaunchEncodeKernel(int grid, cudaStream_t stream, const Job& job, const LevelTables& T0, const LevelTables& T1)
{
	KEncode<kD, NORMAL, SHAPE><<<grid, kWarpsPerCta * 32, EncodeSharedBytes<NORMAL>(), stream>>>(job, T0, T1);
	return cudaGetLastError();
}

template<int kD, bool NORMAL, int SHAPE>
cudaError_t EncodeKernelOccupancy(int* ctasPerSm)
{
	const cudaError_t e = PrepareEncodeKernel<kD, NORMAL, SHAPE>();
	if (e != cudaSuccess)
		return e;
	return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctasPerSm, KEncode<kD, NORMAL, SHAPE>, kWarpsPerCta * 32,
		EncodeSharedBytes<NORMAL>());
}

} // namespace nebc7

#define NEBC7_INSTANTIATE_ENCODE(KD, NORMAL, SHAPE) \
	template cudaError_t nebc7::LaunchEncodeKernel<KD, NORMAL, SHAPE>(int, cudaStream_t, const nebc7::Job&, \
		const nebc7::LevelTables&, const nebc7::LevelTables&); \
	template cudaError_t nebc7::EncodeKernelOccupancy<KD, NORMAL, SHAPE>(int*);
