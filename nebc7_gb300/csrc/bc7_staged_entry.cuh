/*
 * Definitions of the staged-encode launchers declared in bc7_staged.cuh;
 * included by the per-kDenoise translation units only.
 */
#pragma once

#include "bc7_staged.cuh"

namespace nebc7 {

/* The rounds of split pass STAGE over the list KStageListByError gathered:
   round r's tasks, then its commit, which fills the next round's list; after
   the last round the blocks still searching run the rest of the pass in
   one warp each (KEncodeStage from their start partitions). */
template<int kD, int STAGE>
cudaError_t LaunchSplitStage(int grid, cudaStream_t stream, const Job& job, const Stages& sg, const LevelTables& T0, const LevelTables& T1)
{
	constexpr int kRounds = SplitRounds(STAGE);
	static_assert(kRounds <= kSplitMaxRounds, "the split counters hold kSplitMaxRounds rounds");
	int* c = sg.split + SplitIndex(STAGE) * kSplitCounterInts;   /* [round][list length, task head, kept results] */
	const int small = job.total < 256 ? 1 : ((job.total + 255) / 256 < 1216 ? (job.total + 255) / 256 : 1216);
	KSplitPrepare<<<small, 256, 0, stream>>>(sg, sg.list, sg.count + STAGE);
	/* round r > 0 reads the list round r - 1's commit wrote: the two round
	   lists alternate */
	for (int r = 0; r < kRounds; r++)
	{
		const int* list = r ? sg.splitList[(r - 1) & 1] : sg.list;
		const int* count = r ? c + 4 * r : sg.count + STAGE;
		const int nSplit = kSplitMaxBlocks;
		KEncodeSplit<kD, STAGE><<<grid, kWarpsPerCta * 32, EncodeSharedBytes<true>(), stream>>>(job, sg, list, count, c + 4 * r + 1,
			c + 4 * r + 2, nSplit, T0, T1);
		const bool last = r == kRounds - 1;
		KSplitCommit<STAGE><<<small, 256, 0, stream>>>(job, sg, list, count, nSplit, last ? nullptr : sg.splitList[r & 1],
			last ? nullptr : c + 4 * (r + 1), sg.splitList[2], c + 4 * kSplitMaxRounds, int(last));
	}
	KEncodeStage<kD, STAGE><<<grid, kWarpsPerCta * 32, EncodeSharedBytes<true>(), stream>>>(job, sg, sg.splitList[2],
		c + 4 * kSplitMaxRounds, c + 4 * kSplitMaxRounds + 1, T0, T1);
	return cudaGetLastError();
}

template<int kD, int STAGE>
cudaError_t LaunchStage(int grid, cudaStream_t stream, const Job& job, const Stages& sg, const LevelTables& T0, const LevelTables& T1)
{
	/* the passes after the draft chain take their blocks largest error
	   first; the draft chain and the pack keep the queue order, and so do
	   the passes of a mixed launch, whose queue keeps each texture's blocks
	   (of one kDenoise) together */
	if (kD != kAnyDenoise && STAGE >= kStepRefine && STAGE < kStepFinish)
		KStageListByError<<<1, 1024, 0, stream>>>(sg.next, sg.rec, job.total, STAGE, sg.list, sg.count + STAGE);
	else if (STAGE != kStageDraft)
		KStageList<<<1, 1024, 0, stream>>>(sg.next, job.total, STAGE, sg.list, sg.count + (STAGE < 0 ? 0 : STAGE));
	if constexpr (SplitIndex(STAGE) >= 0)
		return LaunchSplitStage<kD, STAGE>(grid, stream, job, sg, T0, T1);
	else
	{
		const bool all = STAGE == kStageDraft;
		KEncodeStage<kD, STAGE><<<grid, kWarpsPerCta * 32, EncodeSharedBytes<true>(), stream>>>(job, sg, all ? nullptr : sg.list,
			all ? nullptr : sg.count + STAGE, sg.counters + (STAGE + 1), T0, T1);
		return cudaGetLastError();
	}
}

template<int kD>
cudaError_t LaunchStagedEncode(int grid, cudaStream_t stream, const Job& job, const Stages& sg, const LevelTables& T0,
	const LevelTables& T1)
{
	cudaError_t e = LaunchStage<kD, kStageDraft>(grid, stream, job, sg, T0, T1);
	if (e == cudaSuccess) e = LaunchStage<kD, kStepDraftRot>(grid, stream, job, sg, T0, T1);
	if (e == cudaSuccess) e = LaunchStage<kD, kStepDraftMode7>(grid, stream, job, sg, T0, T1);
	if (e == cudaSuccess) e = LaunchStage<kD, kStepDraftOpaque31>(grid, stream, job, sg, T0, T1);
	if (e == cudaSuccess) e = LaunchStage<kD, kStepDraftOpaque20>(grid, stream, job, sg, T0, T1);
	if (e == cudaSuccess) e = LaunchStage<kD, kStepRefine>(grid, stream, job, sg, T0, T1);
	if (e == cudaSuccess) e = LaunchStage<kD, kStepFull3Mode2>(grid, stream, job, sg, T0, T1);
	if (e == cudaSuccess) e = LaunchStage<kD, kStepFull3Mode0>(grid, stream, job, sg, T0, T1);
	if (e == cudaSuccess) e = LaunchStage<kD, kStepFull2Mode1>(grid, stream, job, sg, T0, T1);
	if (e == cudaSuccess) e = LaunchStage<kD, kStepFull2Mode3>(grid, stream, job, sg, T0, T1);
	if (e == cudaSuccess) e = LaunchStage<kD, kStepRot5>(grid, stream, job, sg, T0, T1);
	if (e == cudaSuccess) e = LaunchStage<kD, kStepRot4>(grid, stream, job, sg, T0, T1);
	if (e == cudaSuccess) e = LaunchStage<kD, kStepMode7>(grid, stream, job, sg, T0, T1);
	if (e == cudaSuccess) e = LaunchStage<kD, kStepMode6>(grid, stream, job, sg, T0, T1);
	if (e == cudaSuccess) e = LaunchStage<kD, kStepFinish>(grid, stream, job, sg, T0, T1);
	return e;
}

template<int kD, int STAGE>
cudaError_t PrepareStage()
{
	const cudaError_t e = cudaFuncSetAttribute(KEncodeStage<kD, STAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		int(EncodeSharedBytes<true>()));
	if constexpr (SplitIndex(STAGE) >= 0)
		if (e == cudaSuccess)
			return cudaFuncSetAttribute(KEncodeSplit<kD, STAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(EncodeSharedBytes<true>()));
	return e;
}

template<int kD>
cudaError_t StagedEncodeOccupancy(int* ctasPerSm)
{
	cudaError_t e = PrepareStage<kD, kStageDraft>();
	if (e == cudaSuccess) e = PrepareStage<kD, kStepDraftRot>();
	if (e == cudaSuccess) e = PrepareStage<kD, kStepDraftMode7>();
	if (e == cudaSuccess) e = PrepareStage<kD, kStepDraftOpaque31>();
	if (e == cudaSuccess) e = PrepareStage<kD, kStepDraftOpaque20>();
	if (e == cudaSuccess) e = PrepareStage<kD, kStepRefine>();
	if (e == cudaSuccess) e = PrepareStage<kD, kStepFull3Mode2>();
	if (e == cudaSuccess) e = PrepareStage<kD, kStepFull3Mode0>();
	if (e == cudaSuccess) e = PrepareStage<kD, kStepFull2Mode1>();
	if (e == cudaSuccess) e = PrepareStage<kD, kStepFull2Mode3>();
	if (e == cudaSuccess) e = PrepareStage<kD, kStepRot5>();
	if (e == cudaSuccess) e = PrepareStage<kD, kStepRot4>();
	if (e == cudaSuccess) e = PrepareStage<kD, kStepMode7>();
	if (e == cudaSuccess) e = PrepareStage<kD, kStepMode6>();
	if (e == cudaSuccess) e = PrepareStage<kD, kStepFinish>();
	if (e != cudaSuccess)
		return e;
	/* every stage kernel has the refining kernel's shared memory and bounds */
	return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctasPerSm, KEncodeStage<kD, kStepFull3Mode2>, kWarpsPerCta * 32,
		EncodeSharedBytes<true>());
}

} // namespace nebc7

#define NEBC7_INSTANTIATE_STAGED(KD) \
	template cudaError_t nebc7::LaunchStagedEncode<KD>(int, cudaStream_t, const nebc7::Job&, const nebc7::Stages&, \
		const nebc7::LevelTables&, const nebc7::LevelTables&); \
	template cudaError_t nebc7::StagedEncodeOccupancy<KD>(int*);
