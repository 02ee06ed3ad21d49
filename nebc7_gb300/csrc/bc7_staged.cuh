/*
 * BC7 block encoder for sm_103a -- the staged encode of the presets whose
 * time goes to the full searches (precise, /slow, /data, mixed batches).
 *
 * The per-block pipeline of src/Bc7Core.cpp:1516-1823 runs as a sequence of
 * persistent kernels instead of one: the start of the draft chain (the
 * starting block, the Mode6Index2 and mode 6 fast passes), the rest of the
 * draft chain in four kernels, one kernel per refinement / full-search pass
 * of the normal and slow chains (src/Bc7Core.cpp:1604-1745), then the final
 * pack, self-check and quality sums.  Every kernel holds the code of one or
 * two passes, so the warps of an SM run the same few kilobytes of
 * instructions; in a single kernel whose warps
 * sit in different passes the instruction working set outgrows the
 * instruction cache and most issue slots are lost to instruction fetch.
 *
 * Between kernels a block's state (the reference's Cell scalars: best
 * endpoints, mode, partition, errors, stepping values, the starting block)
 * is kept in a BlockRecord per queue position; the pixel data and the
 * whole-block area are rebuilt from the texture when a pass starts.  Each
 * pass kernel runs the blocks whose next pass it is, gathered by
 * KStageList (queue order) or KStageListByError (largest error first).
 * The passes, their order and their entry conditions are those of
 * NormalPasses, so the blocks are the same bits as the single-kernel
 * encode's.
 *
 * The full searches of modes 1, 3 and 7 (64 two-subset partitions each)
 * and of modes 4 and 5 (8 and 4 rotation / index-size choices) are split
 * passes: a few hard blocks take most of their time, and one warp per block
 * would leave the GPU waiting for them.  A split pass runs in rounds.  In a
 * round every candidate (partition or rotation) of every block in the
 * round's list is a task of its own, taken by any warp, searched from the
 * block's error at the start of the round.  The candidates before a block's
 * first improving candidate f searched from that error, as the reference's
 * loop does, so their verdicts stand; f's result is the reference's too.
 * The round's commit applies f and ends the pass, or the block continues
 * in the next round from candidate f + 1 with the new error.  Improvements
 * are rare, so most blocks finish in the first round; blocks still
 * searching after SplitRounds(S) rounds finish their pass in one warp each.
 */
#pragma once

#include "bc7_encode.cuh"

namespace nebc7 {

/* The passes after the first kernel, in chain order: the rest of the draft
   chain, then the normal and slow chains; kStepFinish packs. */
enum StageStep
{
	kStepDraftRot = 0,     /* fast passes of modes 4 and 5 */
	kStepDraftMode7,       /* fast pass of mode 7 */
	kStepDraftOpaque31,    /* fast passes of the opaque modes 3 and 1 */
	kStepDraftOpaque20,    /* fast passes of the opaque modes 2 and 0 */
	kStepRefine,
	kStepFull3Mode2,
	kStepFull3Mode0,
	kStepFull2Mode1,
	kStepFull2Mode3,
	kStepRot5,
	kStepRot4,
	kStepMode7,
	kStepMode6,
	kStepFinish,
	kNumStages
};

constexpr int kStageDraft = -1;
constexpr int kStepNone = -1;   /* finished in the first kernel (an exact starting block) */

/* A block's Cell scalars between pass kernels. */
struct __align__(16) BlockRecord
{
	Ep best[3];
	uint64_t startLo, startHi;   /* the starting block (self-check fallback) */
	int bestParam, bestMode, opaqueAlphaError, errAlpha;
	int errTotal, personalParam, personalMode, denoiseStep;
	int water;                   /* the error at the start of the draft chain */
	int opaque;                  /* the whole-block area's opaque flag */
	int pad[2];
};

/* An improving candidate of a split pass: its endpoints, error and
   parameter (partition or rotation), and whether it ends the full search
   (src/Bc7CoreMode1.cpp:563-564, src/Bc7CoreMode7.cpp:719-720,
   src/Bc7CoreMode4.cpp:1852-1853). */
struct __align__(16) SplitResult
{
	Ep best0, best1;
	int error, end, param;
	int pad;
};

/* The split passes and their rounds. */
constexpr int kSplitMaxRounds = 8;
constexpr int kSplitMaxBlocks = 1 << 24;    /* blocks of a round split into partition tasks (the task count stays an int) */
constexpr int kSplitSerial = -1;            /* firstImp: the block's pass runs whole (OPTION_PCA) */
constexpr int kSplitNone = 0x7FFFFFFF;      /* firstImp: no improvement yet */

__host__ __device__ constexpr int SplitIndex(int S)
{
	return S == kStepFull2Mode1 ? 0 : (S == kStepFull2Mode3 ? 1 : (S == kStepRot5 ? 2 : (S == kStepRot4 ? 3 : (S == kStepMode7 ? 4 : -1))));
}

/* Candidates (tasks) per block of split pass S, and its mode. */
__host__ __device__ constexpr int SplitTasks(int S)
{
	return S == kStepRot4 ? 8 : (S == kStepRot5 ? 4 : 64);
}

__host__ __device__ constexpr int SplitMode(int S)
{
	return S == kStepFull2Mode1 ? 1 : (S == kStepFull2Mode3 ? 3 : (S == kStepRot5 ? 5 : (S == kStepRot4 ? 4 : 7)));
}

/* Rounds of split pass S: one per candidate for the rotation searches,
   whose choices often improve one after another; three for the partition
   searches, where a block rarely improves more than twice. */
__host__ __device__ constexpr int SplitRounds(int S)
{
	return S == kStepRot4 || S == kStepRot5 ? SplitTasks(S) : 3;
}

/* Kernel launches of one staged encode: the draft kernel, then per pass its
   list and its kernel, or for a split pass its list, the preparation, a
   task and a commit kernel per round and the one-warp rest. */
__host__ __device__ constexpr int StagedLaunches()
{
	int n = 1;
	for (int S = 0; S < kNumStages; S++)
		n += SplitIndex(S) >= 0 ? 3 + 2 * SplitRounds(S) : 2;
	return n;
}

/* Ints of the zeroed split counters per split pass: [round][list length,
   task head, kept results, unused], the last row for the one-warp rest. */
constexpr int kSplitCounterInts = 4 * (kSplitMaxRounds + 1);

/* Per-launch state of a staged encode (one entry per queue position). */
struct Stages
{
	BlockRecord* rec;
	int* next;        /* the pass a position waits for, kStepFinish, or kStepNone */
	int* list;        /* positions of the pass being run, in queue order */
	int* count;       /* [kNumStages] list lengths */
	int* counters;    /* [kNumStages + 1] work-queue heads, zero before the draft kernel */
	/* split passes */
	int* start;       /* per position: the first candidate of the block's next round */
	int* firstImp;    /* per position: (candidate << 24) | result slot of the round's first improvement */
	int* splitList[3];   /* the lists of the later rounds (alternately) and of the one-warp remainder */
	int* split;       /* [5 split passes][kSplitCounterInts] list lengths, task heads, result counts; zero before the draft kernel */
	SplitResult* imp;
	int impCap;
};

__device__ __forceinline__ void SaveRecord(BlockRecord& r, const CellRegs& R, int lane)
{
	if (lane == 0)
	{
		r.best[0] = R.best[0];
		r.best[1] = R.best[1];
		r.best[2] = R.best[2];
		r.bestParam = R.bestParam;
		r.bestMode = R.bestMode;
		r.opaqueAlphaError = R.opaqueAlphaError;
		r.errAlpha = R.errAlpha;
		r.errTotal = R.errTotal;
		r.personalParam = R.personalParam;
		r.personalMode = R.personalMode;
		r.denoiseStep = R.denoiseStep;
		r.opaque = R.a1.opaque;
	}
}

/* Rebuilds a block's state: its pixels and masks, the saved scalars, the
   whole-block area (src/Bc7Core.cpp:1532-1535). */
__device__ __forceinline__ void RestoreBlock(WarpState& st, CellRegs& R, const BlockRef& b, const BlockRecord& r, const Params& P,
	int lane)
{
	LoadCell(st, b, R, lane);
	R.best[0] = r.best[0];
	R.best[1] = r.best[1];
	R.best[2] = r.best[2];
	R.bestParam = r.bestParam;
	R.bestMode = r.bestMode;
	R.opaqueAlphaError = r.opaqueAlphaError;
	R.errAlpha = r.errAlpha;
	R.errTotal = r.errTotal;
	R.personalParam = r.personalParam;
	R.personalMode = r.personalMode;
	R.denoiseStep = r.denoiseStep;
	R.a1 = AreaStats(st, R, P, 0xFFFF);
	R.a1.zero = 0;
	BuildAreaList(st.area1, st, R, 0xFFFF, 0, lane);
}

/* One stage: passes of the draft chain after the mode 6 fast pass
   (DraftChain), or one pass of the normal / slow chains (NormalPasses). */
template<int kD, int S>
__device__ __forceinline__ void RunStep(WarpState& st, SearchState& ss, CellRegs& R, const Params& P, const LevelTables& T, int lane,
	int from = 0)
{
	if constexpr (S == kStepDraftRot)
	{
		/* entered with errTotal > step (src/Bc7Core.cpp:1558-1566) */
		FastRot<kD, 4>(st, R, P, lane);
		if (R.errTotal > R.denoiseStep)
			FastRot<kD, 5>(st, R, P, lane);
	}
	else if constexpr (S == kStepDraftMode7)
		FastMode7<kD>(st, R, P, T, lane);
	else if constexpr (S == kStepDraftOpaque31)
	{
		/* entered with errTotal > OA + step (src/Bc7Core.cpp:1577-1585) */
		FastOpaque<kD, 3>(st, R, P, lane);
		if (R.errTotal > R.opaqueAlphaError + R.denoiseStep)
			FastOpaque<kD, 1>(st, R, P, lane);
	}
	else if constexpr (S == kStepDraftOpaque20)
	{
		FastOpaque<kD, 2>(st, R, P, lane);
		if (R.errTotal > R.opaqueAlphaError + R.denoiseStep)
			FastOpaque<kD, 0>(st, R, P, lane);
	}
	else if constexpr (S == kStepRefine)
	{
		const int OA = R.opaqueAlphaError;
		switch (R.bestMode)
		{
		case 0: if (R.errTotal > OA) RefineOpaque<kD, 0>(st, ss, R, P, T, lane); break;
		case 1: if (R.errTotal > OA) RefineOpaque<kD, 1>(st, ss, R, P, T, lane); break;
		case 2: if (R.errTotal > OA) RefineOpaque<kD, 2>(st, ss, R, P, T, lane); break;
		case 3: if (R.errTotal > OA) RefineOpaque<kD, 3>(st, ss, R, P, T, lane); break;
		case 4: if (R.errTotal > 0) RefineMode4<kD>(st, ss, R, P, T, lane); break;
		case 5: if (R.errTotal > 0) RefineMode5<kD>(st, ss, R, P, T, lane); break;
		case 6: if (R.errTotal > 0) RefineMode6<kD, 6>(st, ss, R, P, T, lane); break;
		case 7: if (R.errTotal > 0) RefineMode7<kD>(st, ss, R, P, T, lane); break;
		case 9: if (R.errTotal > 0) RefineMode6<kD, 9>(st, ss, R, P, T, lane); break;
		}
		R.personalParam = R.bestParam;
		R.personalMode = R.bestMode;
	}
	else if constexpr (S == kStepFull3Mode2)
		FullThreeSubsets<kD, 2>(st, ss, R, P, T, lane);
	else if constexpr (S == kStepFull3Mode0)
		FullThreeSubsets<kD, 0>(st, ss, R, P, T, lane);
	else if constexpr (S == kStepFull2Mode1)
		FullTwoSubsets<kD, 1>(st, ss, R, P, T, lane, from);
	else if constexpr (S == kStepFull2Mode3)
		FullTwoSubsets<kD, 3>(st, ss, R, P, T, lane, from);
	else if constexpr (S == kStepRot5)
		FullRot<kD, 5>(st, ss, R, P, T, lane, from);
	else if constexpr (S == kStepRot4)
		FullRot<kD, 4>(st, ss, R, P, T, lane, from);
	else if constexpr (S == kStepMode7)
		FullMode7<kD>(st, ss, R, P, T, lane, from);
	else if constexpr (S == kStepMode6)
		FullMode6<kD>(st, ss, R, P, T, lane);
}

/* The draft chain's opaque passes run for blocks whose alpha stays above
   239 (src/Bc7Core.cpp:1577), after the transparent chain however far it
   went; then the normal passes, or the pack. */
__device__ __forceinline__ int AfterTransparentChain(const CellRegs& R, const Params& P)
{
	if (int(int16_t(R.a1.minmax[0])) > 255 - 16 && R.errTotal > R.opaqueAlphaError + R.denoiseStep)
		return kStepDraftOpaque31;
	return (P.doNormal && P.doDraft != 2) ? kStepRefine : kStepFinish;
}

/* The pass after S: the nesting of the draft chain (src/Bc7Core.cpp:
   1546-1597, DraftChain) and of the normal and slow chains in NormalPasses
   (src/Bc7Core.cpp:1677-1745), whose conditions are tested when each pass
   is reached. */
__device__ __forceinline__ int NextStep(int S, const CellRegs& R, const Params& P)
{
	const int OA = R.opaqueAlphaError, step = R.denoiseStep, e = R.errTotal;
	const int afterDraft = (P.doNormal && P.doDraft != 2) ? kStepRefine : kStepFinish;
	switch (S)
	{
	case kStepDraftRot: return e > step ? kStepDraftMode7 : AfterTransparentChain(R, P);
	case kStepDraftMode7: return AfterTransparentChain(R, P);
	case kStepDraftOpaque31: return e > OA + step ? kStepDraftOpaque20 : afterDraft;
	case kStepDraftOpaque20: return afterDraft;
	default: break;
	}
	if (R.a1.opaque)
	{
		switch (S)
		{
		case kStepRefine: return e > OA + step ? kStepFull3Mode2 : kStepFinish;
		case kStepFull3Mode2: return e > OA + step ? kStepFull3Mode0 : kStepFinish;
		case kStepFull3Mode0: return (P.doSlow && e > OA + step) ? kStepFull2Mode1 : kStepFinish;
		case kStepFull2Mode1: return e > OA + step ? kStepFull2Mode3 : kStepFinish;
		case kStepFull2Mode3: return e > step ? kStepRot5 : kStepFinish;
		case kStepRot5: return e > step ? kStepRot4 : kStepFinish;
		case kStepRot4: return e > step ? kStepMode7 : kStepFinish;
		case kStepMode7: return e > step ? kStepMode6 : kStepFinish;
		default: return kStepFinish;
		}
	}
	switch (S)
	{
	case kStepRefine: return e > step ? kStepRot5 : kStepFinish;
	case kStepRot5: return e > step ? kStepRot4 : kStepFinish;
	case kStepRot4: return e > step ? kStepMode7 : kStepFinish;
	case kStepMode7: return (P.doSlow && e > step) ? kStepMode6 : kStepFinish;
	default: return kStepFinish;
	}
}

/* Writes the block and its result (src/Bc7Core.cpp:1976-1984). */
template<int kD>
__device__ __forceinline__ void StoreBlock(const BlockRef& b, const CellRegs& R, uint64_t lo, uint64_t hi, double qa, double qc,
	int lane)
{
	if (lane == 0)
	{
		*reinterpret_cast<uint4*>(b.out) = make_uint4(unsigned(lo), unsigned(lo >> 32), unsigned(hi), unsigned(hi >> 32));
		if (b.result)
		{
			BlockResult r;
			r.errAlpha = int(unsigned(R.errAlpha) << (kD + kD));
			r.errColor = int(unsigned(R.errTotal - R.errAlpha) << (kD + kD));
			r.ssimAlpha = qa;
			r.ssimColor = qc;
			*b.result = r;
		}
	}
	__syncwarp();
}

/* The final pack when the search beat the starting block, then the
   self-check (src/Bc7Core.cpp:1799-1807) and the SSIM sums. */
template<int kD>
__device__ __forceinline__ void FinishBlock(WarpState& st, CellRegs& R, const Params& P, int water, uint64_t startLo, uint64_t startHi,
	const BlockRef& b, int lane)
{
	uint64_t lo = startLo, hi = startHi;
	if (water > R.errTotal)
		FinalPack<kD>(st, R, P, lo, hi, lane);
	Ep dummy[3];
	int dp, dm;
	DecodeToState(st, lo, hi, dummy, dp, dm, lane);
	int ea, et;
	CompareBlocks<kD>(st, P, lane, ea, et);
	if (ea != R.errAlpha || et != R.errTotal)
	{
		lo = startLo;
		hi = startHi;
	}
	double qa = 1.0, qc = 1.0;
	CompareBlocksSSIM(st, P, lane, qa, qc);
	StoreBlock<kD>(b, R, lo, hi, qa, qc, lane);
}

/* The first kernel's block: the start of EncodeBlockAt and of the draft
   chain (src/Bc7Core.cpp:1516-1556: the starting block, its error, the
   stepping values, the Mode6Index2 and mode 6 fast passes).  An exact
   starting block is written at once; every other block saves its record
   for the next stage and waits.  Returns whether the block finished. */
template<int kD>
__device__ bool DraftStage(WarpState& st, const BlockRef& b, const LevelTables& T, const Params& P, BlockRecord& rec, int& next,
	int lane)
{
	CellRegs R;
	LoadCell(st, b, R, lane);
	const uint4 blk = *reinterpret_cast<const uint4*>(b.out);
	uint64_t lo = uint64_t(blk.x) | (uint64_t(blk.y) << 32);
	uint64_t hi = uint64_t(blk.z) | (uint64_t(blk.w) << 32);
	if (!(lo & 0xFF))
	{
		/* src/Bc7Core.cpp:1518-1522: an empty block starts as a zero mode 6 block */
		lo = 1u << 6;
		hi = 0;
	}
	DecodeToState(st, lo, hi, R.best, R.bestParam, R.bestMode, lane);
	CompareBlocks<kD>(st, P, lane, R.errAlpha, R.errTotal);
	if (!(R.errTotal > 0))
	{
		StoreBlock<kD>(b, R, lo, hi, 1.0, 1.0, lane);
		if (lane == 0)
			next = kStepNone;
		return true;
	}
	R.a1 = AreaStats(st, R, P, 0xFFFF);
	R.a1.zero = 0;
	BuildAreaList(st.area1, st, R, 0xFFFF, 0, lane);
	R.personalMode = -1;
	R.personalParam = -1;
	const int water = R.errTotal;
	int n = kStepFinish;
	if (P.doDraft)
	{
		const int step = R.a1.active * ((P.denoiseStep * (R.a1.opaque ? P.wColor : P.wColorAlpha)) >> (kD + kD));
		R.denoiseStep = step;
		/* src/Bc7Core.cpp:24-50 */
		{
			int e = 0;
			if (!R.a1.opaque && lane < 16)
			{
				int da = int(st.area1.px[lane][0]) ^ 255;
				da = kD ? (da >> kD) : (da > 0x7F ? 0x7F : da);
				e = da * da;
			}
			e = int(__reduce_add_sync(kFull, unsigned(e)));
			R.opaqueAlphaError = R.a1.opaque ? 0 : e * P.wA;
		}
		if (P.doDraft == 2)
		{
			/* the "Mode6Index2 fast" run: the draft chain reduced to its
			   first pass (no counterpart in the reference) */
			if (R.errTotal > step && (kD > 0 || P.denoiseStep > 0))
				FastMode6<kD, true>(st, R, P, T);
		}
		else
		{
			if (R.errTotal > step)
			{
				if (kD > 0 || P.denoiseStep > 0)
					FastMode6<kD, true>(st, R, P, T);
				if (R.errTotal > step)
				{
					FastMode6<kD, false>(st, R, P, T);
					if (R.errTotal > step)
						n = kStepDraftRot;
				}
			}
			if (n != kStepDraftRot)
				n = AfterTransparentChain(R, P);
		}
	}
	else
	{
		/* no draft chain: the starting block stands (water == errTotal) */
		R.denoiseStep = 0;
		R.opaqueAlphaError = 0;
	}
	SaveRecord(rec, R, lane);
	if (lane == 0)
	{
		rec.startLo = lo;
		rec.startHi = hi;
		rec.water = water;
		next = n;
	}
	__syncwarp();
	return false;
}

/* A pass kernel's block: runs pass S (of a split pass, the partitions from
   `from` on) and records the next one. */
template<int kD, int S>
__device__ void PassStage(WarpState& st, SearchState& ss, const BlockRef& b, const LevelTables& T, const Params& P, BlockRecord& rec,
	int& next, int from, int lane)
{
	CellRegs R;
	RestoreBlock(st, R, b, rec, P, lane);
	RunStep<kD, S>(st, ss, R, P, T, lane, from);
	const int n = NextStep(S, R, P);
	SaveRecord(rec, R, lane);
	if (lane == 0)
		next = n;
	__syncwarp();
}

/* The finish kernel's block. */
template<int kD>
__device__ void FinishStage(WarpState& st, const BlockRef& b, const Params& P, const BlockRecord& rec, int lane)
{
	CellRegs R;
	RestoreBlock(st, R, b, rec, P, lane);
	FinishBlock<kD>(st, R, P, rec.water, rec.startLo, rec.startHi, b, lane);
}

/* Stage STAGE of one block at queue position k; returns whether the block
   finished (its output is written). */
template<int kD, int STAGE>
__device__ __forceinline__ bool StageBlock(WarpState& st, SearchState& ss, const BlockRef& b, const LevelTables& T, const Params& P,
	const Stages& sg, int k, int lane)
{
	if constexpr (STAGE == kStageDraft)
		return DraftStage<kD>(st, b, T, P, sg.rec[k], sg.next[k], lane);
	else if constexpr (STAGE == kStepFinish)
	{
		FinishStage<kD>(st, b, P, sg.rec[k], lane);
		return true;
	}
	else
	{
		PassStage<kD, STAGE>(st, ss, b, T, P, sg.rec[k], sg.next[k], SplitIndex(STAGE) >= 0 ? sg.start[k] : 0, lane);
		return false;
	}
}

/* One stage of a staged encode over a list of queue positions (`list`,
   *count entries, taken through *head): the draft kernel takes every
   position (no list); a pass or the finish kernel takes the positions
   gathered for it.  kD as for KEncode. */
template<int kD, int STAGE>
__global__ void __launch_bounds__(kWarpsPerCta * 32, 4) KEncodeStage(Job job, Stages sg, const int* list, const int* count, int* head,
	LevelTables T0, LevelTables T1)
{
	extern __shared__ __align__(16) unsigned char encodeSmem[];
	const int lane = threadIdx.x & 31;
	const int warp = threadIdx.x >> 5;
	WarpState& st = reinterpret_cast<WarpState*>(encodeSmem)[warp];
	SearchState& ss = reinterpret_cast<SearchState*>(encodeSmem + kWarpsPerCta * sizeof(WarpState))[warp];
	const int n = list ? *count : job.total;
	for (;;)
	{
		int i = 0;
		if (lane == 0)
			i = atomicAdd(head, 1);
		i = __shfl_sync(kFull, i, 0);
		if (i >= n)
			break;
		const int k = list ? list[i] : i;
		TexDesc d;
		BlockRef b;
		QueuedBlock(job, k, d, b);
		const Params P = d.P;
		bool finished;
		if constexpr (kD == kAnyDenoise)
		{
			if (d.denoise)
				finished = StageBlock<1, STAGE>(st, ss, b, T1, P, sg, k, lane);
			else
				finished = StageBlock<0, STAGE>(st, ss, b, T0, P, sg, k, lane);
		}
		else
			finished = StageBlock<kD, STAGE>(st, ss, b, kD ? T1 : T0, P, sg, k, lane);
		if (finished)
			BlockFinished(d, lane);
	}
}

/* One task of a split pass: candidate p of the block at position k,
   searched from the error in its record (the error at the start of the
   round).  An improving candidate before the round's first improvement so
   far keeps its result and lowers the block's firstImp; a candidate after
   it is not searched (the next round searches it again). */
template<int kD, int S>
__device__ NEBC7_PASS void SplitTask(WarpState& st, SearchState& ss, const BlockRef& b, const LevelTables& T, const Params& P,
	const Stages& sg, int* impCount, int k, int p, int lane)
{
	constexpr int MODE = SplitMode(S);
	volatile int* first = sg.firstImp + k;
	/* one read for the whole warp: other warps lower it meanwhile */
	int firstNow = 0;
	if (lane == 0)
		firstNow = *first;
	if ((__shfl_sync(kFull, firstNow, 0) >> 24) < p)
		return;
	CellRegs R;
	RestoreBlock(st, R, b, sg.rec[k], P, lane);
	const int E = R.errTotal, step = R.denoiseStep;
	bool end;
	int param = p;
	/* the conditions of the candidate loops (FullTwoSubsets, FullMode7, FullRot) */
	if constexpr (MODE == 4 || MODE == 5)
	{
		const int rotation = MODE == 4 ? c_rot4[p] : c_rot5[p];
		if (MODE == 4 && R.personalMode == 4 && !((R.personalParam ^ rotation) & 3))
			return;
		if (MODE == 5 && R.personalMode == 5 && R.personalParam == rotation)
			return;
		Ep mc = 0;
		int error = step;
		if (error < E)
			error += CompressRotSubset<kD, MODE>(st, ss, R, P, T, mc, E - error, rotation, lane);
		if (!(E > error))
			return;
		R.errTotal = error - step;
		R.best[0] = mc;
		end = error <= step;
		param = rotation;
	}
	else
	{
		if (R.personalMode == MODE && R.personalParam == p)
			return;
		if constexpr (MODE == 7)
		{
			if (!(0 < E - step) || !(step < E))
				return;
			end = Mode7Partition<kD>(st, ss, R, P, T, p, 0, 0, lane);
		}
		else
		{
			const int OA = R.opaqueAlphaError;
			if (!(0 < E - step - OA) || !(OA + step < E))
				return;
			end = TwoSubsetsPartition<kD, MODE>(st, ss, R, P, GetSpec3<MODE>(T), T, p, 0, 0, lane);
		}
		if (R.errTotal == E)
			return;
	}
	if (lane != 0 || (*first >> 24) < p)
		return;
	int slot = 0xFFFFFF;
	const int at = atomicAdd(impCount, 1);
	if (at < sg.impCap)
	{
		SplitResult r;
		r.best0 = R.best[0];
		r.best1 = R.best[1];
		r.error = R.errTotal;
		r.end = end;
		r.param = param;
		r.pad = 0;
		sg.imp[at] = r;
		slot = at;
	}
	atomicMin(sg.firstImp + k, (p << 24) | slot);
}

/* A round of split pass S over the blocks list[i], i < *count: the first
   nSplit blocks as tasks (block, candidate p) for p from the block's start
   candidate, taken through *head block by block, so that the candidates of
   a block go to as many warps; the blocks after them (with more blocks than
   the task count can number) as one task each, the whole pass in one warp
   (PassStage). */
template<int kD, int S>
__global__ void __launch_bounds__(kWarpsPerCta * 32, 4) KEncodeSplit(Job job, Stages sg, const int* list, const int* count, int* head,
	int* impCount, int nSplit, LevelTables T0, LevelTables T1)
{
	constexpr int NT = SplitTasks(S);
	extern __shared__ __align__(16) unsigned char encodeSmem[];
	const int lane = threadIdx.x & 31;
	const int warp = threadIdx.x >> 5;
	WarpState& st = reinterpret_cast<WarpState*>(encodeSmem)[warp];
	SearchState& ss = reinterpret_cast<SearchState*>(encodeSmem + kWarpsPerCta * sizeof(WarpState))[warp];
	const int n = *count;
	const int heavy = n < nSplit ? n : nSplit;
	for (;;)
	{
		int t = 0;
		if (lane == 0)
			t = atomicAdd(head, 1);
		t = __shfl_sync(kFull, t, 0);
		if (t >= heavy * NT)
		{
			const int i = heavy + (t - heavy * NT);
			if (i >= n)
				break;
			const int k = list[i];
			TexDesc d;
			BlockRef b;
			QueuedBlock(job, k, d, b);
			const Params P = d.P;
			if constexpr (kD == kAnyDenoise)
			{
				if (d.denoise)
					PassStage<1, S>(st, ss, b, T1, P, sg.rec[k], sg.next[k], sg.start[k], lane);
				else
					PassStage<0, S>(st, ss, b, T0, P, sg.rec[k], sg.next[k], sg.start[k], lane);
			}
			else
				PassStage<kD, S>(st, ss, b, kD ? T1 : T0, P, sg.rec[k], sg.next[k], sg.start[k], lane);
			continue;
		}
		const int i = t / NT, p = t % NT;
		const int k = list[i];
		if (p < sg.start[k])
			continue;
		TexDesc d;
		BlockRef b;
		QueuedBlock(job, k, d, b);
		const Params P = d.P;
		if (P.pca && SplitMode(S) != 4 && SplitMode(S) != 5)
		{
			/* OPTION_PCA orders the partitions by their bounds first: the
			   pass runs whole, in one warp */
			if (p == 0 && lane == 0)
				sg.firstImp[k] = kSplitSerial;
			__syncwarp();
			continue;
		}
		if constexpr (kD == kAnyDenoise)
		{
			if (d.denoise)
				SplitTask<1, S>(st, ss, b, T1, P, sg, impCount, k, p, lane);
			else
				SplitTask<0, S>(st, ss, b, T0, P, sg, impCount, k, p, lane);
		}
		else
			SplitTask<kD, S>(st, ss, b, kD ? T1 : T0, P, sg, impCount, k, p, lane);
	}
}

/* Before the first round of a split pass: every block starts at candidate 0
   with no improvement. */
static __global__ void __launch_bounds__(256) KSplitPrepare(Stages sg, const int* list, const int* count)
{
	const int n = *count;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const int k = list[i];
		sg.start[k] = 0;
		sg.firstImp[k] = kSplitNone;
	}
}

/* The commit of a round of split pass S, one thread per split block: the
   first improving candidate f becomes the block's best and ends the pass,
   or the block goes on from f + 1 in the next round's list (after the last
   round, in the one-warp remainder's list); a block without an improvement
   has finished the pass and gets its next one (NextStep). */
template<int S>
__global__ void __launch_bounds__(256) KSplitCommit(Job job, Stages sg, const int* list, const int* count, int nSplit, int* nextList,
	int* nextCount, int* restList, int* restCount, int lastRound)
{
	constexpr int MODE = SplitMode(S);
	/* the blocks after the first nSplit ran their whole pass in one task */
	const int n = *count < nSplit ? *count : nSplit;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const int k = list[i];
		const int f = sg.firstImp[k];
		BlockRecord& r = sg.rec[k];
		if (f == kSplitSerial)
		{
			sg.start[k] = 0;
			restList[atomicAdd(restCount, 1)] = k;
			continue;
		}
		int from = -1;
		if (f != kSplitNone)
		{
			const int p = f >> 24, slot = f & 0xFFFFFF;
			if (slot >= sg.impCap)
				from = p;   /* its result was not kept: search it again */
			else
			{
				const SplitResult e = sg.imp[slot];
				r.errTotal = e.error;
				r.best[0] = e.best0;
				if (MODE != 4 && MODE != 5)
					r.best[1] = e.best1;
				r.bestParam = e.param;
				r.bestMode = MODE;
				if (!e.end && p < SplitTasks(S) - 1)
					from = p + 1;
			}
		}
		if (from >= 0)
		{
			sg.start[k] = from;
			sg.firstImp[k] = kSplitNone;
			if (lastRound)
				restList[atomicAdd(restCount, 1)] = k;
			else
				nextList[atomicAdd(nextCount, 1)] = k;
			continue;
		}
		TexDesc d;
		BlockRef b;
		QueuedBlock(job, k, d, b);
		CellRegs R;
		R.errTotal = r.errTotal;
		R.opaqueAlphaError = r.opaqueAlphaError;
		R.denoiseStep = r.denoiseStep;
		R.a1.opaque = r.opaque != 0;
		sg.next[k] = NextStep(S, R, d.P);
	}
}

/* Gathers, in queue order, the positions whose next pass is `stage` into
   list and their number into *count (one block of 1024 threads, 4096
   positions per round). */
static __global__ void __launch_bounds__(1024) KStageList(const int* next, int total, int stage, int* list, int* count)
{
	__shared__ int warpSums[32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	int base = 0;
	for (int k0 = 0; k0 < total; k0 += 4096)
	{
		const int k = k0 + 4 * int(threadIdx.x);
		bool on[4];
		int mine = 0;
		for (int j = 0; j < 4; j++)
		{
			on[j] = k + j < total && next[k + j] == stage;
			mine += on[j];
		}
		/* inclusive scan of the per-thread counts over the warp, then the block */
		int incl = mine;
		for (int o = 1; o < 32; o <<= 1)
		{
			const int v = __shfl_up_sync(kFull, incl, o);
			if (lane >= o)
				incl += v;
		}
		if (lane == 31)
			warpSums[warp] = incl;
		__syncthreads();
		int before = 0, all = 0;
		for (int w = 0; w < 32; w++)
		{
			const int c = warpSums[w];
			before += w < warp ? c : 0;
			all += c;
		}
		int at = base + before + incl - mine;
		for (int j = 0; j < 4; j++)
			if (on[j])
				list[at++] = k + j;
		base += all;
		__syncthreads();
	}
	if (threadIdx.x == 0)
		*count = base;
}

/* Gathers the positions whose next pass is `stage`, largest error first:
   a counting sort on 8 buckets per octave of the record's errTotal (one
   block of 1024 threads).  A search's cost grows with its water, so the
   longest searches of a pass start first and no SM waits at the end of the
   pass behind a late hard block; the order inside a bucket is any, and
   the blocks written are the same either way. */
static __global__ void __launch_bounds__(1024) KStageListByError(const int* next, const BlockRecord* rec, int total, int stage,
	int* list, int* count)
{
	__shared__ int hist[256];
	__shared__ int base[256];
	for (int i = threadIdx.x; i < 256; i += 1024)
		hist[i] = 0;
	__syncthreads();
	auto bucketOf = [&](int k) {
		const unsigned e = unsigned(max(rec[k].errTotal, 0));
		if (!e)
			return 255;
		const int msb = 31 - __clz(e);
		const int frac = int((e >> (msb >= 3 ? msb - 3 : 0)) & 7u);
		return 255 - min(255, msb * 8 + frac);
	};
	for (int k = threadIdx.x; k < total; k += 1024)
		if (next[k] == stage)
			atomicAdd(&hist[bucketOf(k)], 1);
	__syncthreads();
	if (threadIdx.x == 0)
	{
		int run = 0;
		for (int b = 0; b < 256; b++)
		{
			base[b] = run;
			run += hist[b];
		}
		*count = run;
	}
	__syncthreads();
	for (int k = threadIdx.x; k < total; k += 1024)
		if (next[k] == stage)
			list[atomicAdd(&base[bucketOf(k)], 1)] = k;
}

/* Host-side launcher of a staged encode: the draft kernel, then for each
   pass its list and its kernel, then the finish kernel's list and kernel.
   The launches are capturable.  Compiled per kD in encode_*_staged.cu. */
template<int kD>
cudaError_t LaunchStagedEncode(int grid, cudaStream_t stream, const Job& job, const Stages& sg, const LevelTables& T0,
	const LevelTables& T1);

/* Raises the stage kernels' dynamic shared-memory limit (once per process
   and device, before the first launch) and reports CTAs per SM. */
template<int kD>
cudaError_t StagedEncodeOccupancy(int* ctasPerSm);

/* Bytes of the per-position state of a staged encode of n positions
   (records, next-pass words, the pass list, the split passes' start
   partitions, first improvements, round lists and kept results; 256-byte
   aligned pieces), after kStagedZeroed bytes of counts and queue heads that
   must be zero before each launch. */
constexpr size_t kStagedZeroed = 1280;

constexpr size_t SplitResultCap(int n)
{
	return size_t(n) + 256;
}

constexpr size_t StagedScratchBytes(int n)
{
	return kStagedZeroed + ((size_t(n) * sizeof(BlockRecord) + 255) & ~size_t(255)) + ((size_t(n) * 4 + 255) & ~size_t(255)) * 7 +
		SplitResultCap(n) * sizeof(SplitResult);
}

/* Splits a staged scratch (256-byte aligned, StagedScratchBytes(n) bytes). */
inline Stages SplitStaged(uint8_t* p, int n)
{
	Stages s;
	s.count = (int*)p;
	s.counters = (int*)(p + 128);
	s.split = (int*)(p + 256);
	s.rec = (BlockRecord*)(p + kStagedZeroed);
	uint8_t* q = p + kStagedZeroed + ((size_t(n) * sizeof(BlockRecord) + 255) & ~size_t(255));
	const size_t ints = (size_t(n) * 4 + 255) & ~size_t(255);
	s.next = (int*)q;
	s.list = (int*)(q + ints);
	s.start = (int*)(q + 2 * ints);
	s.firstImp = (int*)(q + 3 * ints);
	s.splitList[0] = (int*)(q + 4 * ints);
	s.splitList[1] = (int*)(q + 5 * ints);
	s.splitList[2] = (int*)(q + 6 * ints);
	s.imp = (SplitResult*)(q + 7 * ints);
	s.impCap = int(SplitResultCap(n));
	return s;
}

} // namespace nebc7
