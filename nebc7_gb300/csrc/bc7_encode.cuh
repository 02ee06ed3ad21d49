/*
 * BC7 block encoder for sm_103a -- the per-block scheduler and the encode /
 * decode kernels.
 *
 * KEncode is a persistent kernel: each warp takes the next block index from
 * a global counter and runs the reference's per-block pipeline
 * (src/Bc7Core.cpp:1516-1823 CompressBlock) on it: decode the block already
 * in `dst` (incremental re-encode), measure it, and unless it is exact run
 * the mode chain with error stepping, pack the winner and self-check it.
 * Block costs differ by orders of magnitude (an exact block stops at once, a
 * hard one searches every partition), so blocks are dealt one at a time.
 */
#pragma once

#include "bc7_fast.cuh"
#include "bc7_search.cuh"

namespace nebc7 {

struct BlockResult
{
	int errAlpha;     /* Error.Alpha << 2 kDenoise */
	int errColor;     /* (Error.Total - Error.Alpha) << 2 kDenoise */
	double ssimAlpha, ssimColor;
};

/* One texture of a launch: padded BGRA rows and optional mask rows, its
   blocks in row-major order, and its preset. */
struct TexDesc
{
	uint8_t* dst;            /* 16 bytes per block, read as the starting block */
	const uint8_t* bgra;     /* top-left pixel of block 0 */
	const uint8_t* mask;     /* same layout, A,G,R,B bytes; null = all 0xFF */
	long long stride;        /* bytes between pixel rows */
	int blocksW;             /* blocks per block row */
	int nblocks;
	int first;               /* queue position of its first block */
	int denoise;             /* kDenoise of its preset */
	int id;                  /* caller's index of the texture (batches) */
	BlockResult* results;    /* its per-block results, or null: the launch's array */
	int* remaining;          /* optional: blocks still to finish (request loop) */
	int* doneFlag;           /* set to 1 (host-mapped memory) when remaining reaches 0 */
	Params P;
};

/* Per-launch description: the textures and the shared work queue.  The
   queue deals blocks in texture-table order; a warp finds the texture of a
   queue position by binary search over `first`. */
struct Job
{
	const TexDesc* tex;      /* device table of ntex textures, or null: `single` */
	TexDesc single;
	int ntex;
	int total;               /* blocks over all textures */
	BlockResult* results;    /* optional, one per queue position */
	int* counter;            /* work queue head, zero before launch */
	int* status;             /* set non-zero on an internal limit */
	const int* order;        /* optional: queue position -> block (`single` only) */
};

/* kD template value of the kernel that reads kDenoise from each texture */
constexpr int kAnyDenoise = 2;

constexpr int kWarpsPerCta = 4;

/* Where one block's pixels, mask and 16 output bytes are. */
struct BlockRef
{
	const uint8_t* bgra;     /* top-left pixel of the block */
	const uint8_t* mask;     /* same position in the mask, or null */
	long long stride;        /* bytes between pixel rows */
	uint8_t* out;            /* the block: starting block in, result out */
	BlockResult* result;     /* optional */
};

/* The draft chain (src/Bc7Core.cpp:1537-1597) after the block's stepping
   values are set: the fast passes of modes 6Index2, 6, 4, 5, 7 with error
   stepping, then, for blocks whose alpha stays above 239, the fast passes of
   the opaque modes 3, 1, 2, 0. */
template<int kD>
__device__ __forceinline__ void DraftChain(WarpState& st, CellRegs& R, const Params& P, const LevelTables& T, int lane)
{
	const int step = R.denoiseStep;
	if (P.doDraft == 2)
	{
		/* the "Mode6Index2 fast" run: the draft chain reduced to its
		   first pass (no counterpart in the reference) */
		if (R.errTotal > step && (kD > 0 || P.denoiseStep > 0))
			FastMode6<kD, true>(st, R, P, T);
	}
	else if (R.errTotal > step)
	{
		if (kD > 0 || P.denoiseStep > 0)
			FastMode6<kD, true>(st, R, P, T);
		if (R.errTotal > step)
		{
			FastMode6<kD, false>(st, R, P, T);
			if (R.errTotal > step)
			{
				FastRot<kD, 4>(st, R, P, lane);
				if (R.errTotal > step)
				{
					FastRot<kD, 5>(st, R, P, lane);
					if (R.errTotal > step)
						FastMode7<kD>(st, R, P, T, lane);
				}
			}
		}
	}

	if (P.doDraft != 2 && int(int16_t(R.a1.minmax[0])) > 255 - 16)
	{
		const int gate = R.opaqueAlphaError + step;
		if (R.errTotal > gate)
		{
			FastOpaque<kD, 3>(st, R, P, lane);
			if (R.errTotal > gate)
			{
				FastOpaque<kD, 1>(st, R, P, lane);
				if (R.errTotal > gate)
				{
					FastOpaque<kD, 2>(st, R, P, lane);
					if (R.errTotal > gate)
						FastOpaque<kD, 0>(st, R, P, lane);
				}
			}
		}
	}
}

/* Coalesced load of one block (lanes 0..15 a BGRA pixel each, 16..31 its
   mask), the masked data (src/Bc7Core.cpp:52-86) and the block-wide
   visibility and opacity. */
__device__ __forceinline__ void LoadCell(WarpState& st, const BlockRef& b, CellRegs& R, int lane)
{
	{
		const int i = lane & 15;
		const long long off = (long long)(i >> 2) * b.stride + (i & 3) * 4;
		if (lane < 16)
		{
			const uchar4 p = *reinterpret_cast<const uchar4*>(b.bgra + off);
			st.img[i][0] = p.w;
			st.img[i][1] = p.y;
			st.img[i][2] = p.z;
			st.img[i][3] = p.x;
		}
		else
		{
			uchar4 m = make_uchar4(0xFF, 0xFF, 0xFF, 0xFF);
			if (b.mask)
				m = *reinterpret_cast<const uchar4*>(b.mask + off);
			st.msk[i][0] = m.x;
			st.msk[i][1] = m.y;
			st.msk[i][2] = m.z;
			st.msk[i][3] = m.w;
		}
	}
	__syncwarp();
	uint32_t visBit = 0;
	unsigned alphaAnd = 0xFF;
	if (lane < 16)
	{
		for (int c = 0; c < 4; c++)
		{
			const uint16_t m = uint16_t(int16_t(int8_t(st.msk[lane][c])));
			st.mk[lane][c] = m;
			st.px[lane][c] = uint16_t(st.img[lane][c] & m);
		}
		visBit = (st.mk[lane][1] >> lane) & 1;
		alphaAnd = st.px[lane][0];
	}
	R.visible = __ballot_sync(kFull, visBit != 0) & 0xFFFF;
	R.opaque = __reduce_and_sync(kFull, alphaAnd) == 255;
}

template<int kD, bool NORMAL>
__device__ void EncodeBlockAt(WarpState& st, SearchState* ss, const BlockRef& b, const LevelTables& T, const Params& P, int lane)
{
	/* coalesced load: lanes 0..15 read one BGRA pixel, 16..31 its mask */
	{
		const int i = lane & 15;
		const long long off = (long long)(i >> 2) * b.stride + (i & 3) * 4;
		if (lane < 16)
		{
			const uchar4 p = *reinterpret_cast<const uchar4*>(b.bgra + off);
			st.img[i][0] = p.w;
			st.img[i][1] = p.y;
			st.img[i][2] = p.z;
			st.img[i][3] = p.x;
		}
		else
		{
			uchar4 m = make_uchar4(0xFF, 0xFF, 0xFF, 0xFF);
			if (b.mask)
				m = *reinterpret_cast<const uchar4*>(b.mask + off);
			st.msk[i][0] = m.x;
			st.msk[i][1] = m.y;
			st.msk[i][2] = m.z;
			st.msk[i][3] = m.w;
		}
	}
	const uint4 blk = *reinterpret_cast<const uint4*>(b.out);
	__syncwarp();

	uint64_t lo = uint64_t(blk.x) | (uint64_t(blk.y) << 32);
	uint64_t hi = uint64_t(blk.z) | (uint64_t(blk.w) << 32);
	if (!(lo & 0xFF))
	{
		/* src/Bc7Core.cpp:1518-1522: an empty block starts as a zero mode 6 block */
		lo = 1u << 6;
		hi = 0;
	}
	const uint64_t savedLo = lo, savedHi = hi;

	/* widened masks and masked data (src/Bc7Core.cpp:52-86) */
	uint32_t visBit = 0;
	unsigned alphaAnd = 0xFF;
	if (lane < 16)
	{
		for (int c = 0; c < 4; c++)
		{
			const uint16_t m = uint16_t(int16_t(int8_t(st.msk[lane][c])));
			st.mk[lane][c] = m;
			st.px[lane][c] = uint16_t(st.img[lane][c] & m);
		}
		visBit = (st.mk[lane][1] >> lane) & 1;
		alphaAnd = st.px[lane][0];
	}
	CellRegs R;
	R.visible = __ballot_sync(kFull, visBit != 0) & 0xFFFF;
	R.opaque = __reduce_and_sync(kFull, alphaAnd) == 255;

	DecodeToState(st, lo, hi, R.best, R.bestParam, R.bestMode, lane);
	CompareBlocks<kD>(st, P, lane, R.errAlpha, R.errTotal);

	double qa = 1.0, qc = 1.0;
	if (R.errTotal > 0)
	{
		R.a1 = AreaStats(st, R, P, 0xFFFF);
		R.a1.zero = 0;
		BuildAreaList(st.area1, st, R, 0xFFFF, 0, lane);
		R.personalMode = -1;
		R.personalParam = -1;

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
			const int water = R.errTotal;

			DraftChain<kD>(st, R, P, T, lane);

			if (NORMAL && P.doNormal && P.doDraft != 2)
				NormalPasses<kD>(st, *ss, R, P, T, lane);

			if (water > R.errTotal)
				FinalPack<kD>(st, R, P, lo, hi, lane);
		}

		/* self-check (src/Bc7Core.cpp:1799-1807): the packed block must decode to
		   the tracked error, otherwise the starting block is kept */
		Ep dummy[3];
		int dp, dm;
		DecodeToState(st, lo, hi, dummy, dp, dm, lane);
		int ea, et;
		CompareBlocks<kD>(st, P, lane, ea, et);
		if (ea != R.errAlpha || et != R.errTotal)
		{
			lo = savedLo;
			hi = savedHi;
		}
		CompareBlocksSSIM(st, P, lane, qa, qc);
	}

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

/* Texture and block of queue position k of the launch. */
__device__ __forceinline__ void QueuedBlock(const Job& job, int k, TexDesc& d, BlockRef& b)
{
	if (job.order)
		k = job.order[k];
	int t = 0;
	if (job.tex)
	{
		int hi = job.ntex - 1;
		while (t < hi)
		{
			const int mid = (t + hi + 1) >> 1;
			if (job.tex[mid].first <= k)
				t = mid;
			else
				hi = mid - 1;
		}
	}
	/* a copy, read from the table or from the launch's parameters (no
	   pointer into the parameters, which would put them in local memory) */
	if (job.tex)
		d = job.tex[t];
	else
		d = job.single;
	const int local = k - d.first;
	const int bx = local % d.blocksW, by = local / d.blocksW;
	const long long base = (long long)by * 4 * d.stride + (long long)bx * 16;
	b.bgra = d.bgra + base;
	b.mask = d.mask ? d.mask + base : nullptr;
	b.stride = d.stride;
	b.out = d.dst + (long long)local * 16;
	b.result = d.results ? d.results + local : (job.results ? job.results + k : nullptr);
}

/* Publishes a finished block of a request-loop texture: counts it and lets
   the last one tell the host that the texture is complete. */
__device__ __forceinline__ void BlockFinished(const TexDesc& d, int lane)
{
	if (d.remaining && lane == 0)
	{
		/* lane 0 wrote the block and its result: publish them first */
		__threadfence();
		if (atomicSub(d.remaining, 1) == 1)
		{
			__threadfence_system();
			*reinterpret_cast<volatile int*>(d.doneFlag) = 1;
		}
	}
	__syncwarp();
}

/* Encodes queue position k of the launch. */
template<int kD, bool NORMAL>
__device__ __forceinline__ void EncodeQueued(WarpState& st, SearchState* ss, const Job& job, const LevelTables& T0,
	const LevelTables& T1, int k, int lane)
{
	TexDesc d;
	BlockRef b;
	QueuedBlock(job, k, d, b);
	const Params P = d.P;
	if (kD == kAnyDenoise)
	{
		if (d.denoise)
			EncodeBlockAt<1, NORMAL>(st, ss, b, T1, P, lane);
		else
			EncodeBlockAt<0, NORMAL>(st, ss, b, T0, P, lane);
	}
	else
		EncodeBlockAt<kD == 1 ? 1 : 0, NORMAL>(st, ss, b, kD ? T1 : T0, P, lane);
	BlockFinished(d, lane);
}

/* Dynamic shared memory of one encode CTA: the per-warp block state and,
   for the refining instantiation, the per-warp search state. */
template<bool NORMAL>
constexpr size_t EncodeSharedBytes()
{
	return kWarpsPerCta * (sizeof(WarpState) + (NORMAL ? sizeof(SearchState) : 0));
}

/* Code shapes of the refining kernel.  Compact: every routine inlined (the
   fastest for the default preset, whose time goes to one refinement).
   Outlined: the routines the full searches call from many places kept out
   of line (NEBC7_SHARED) and registers bounded for 4 CTAs per SM (the
   fastest for the precise preset, /slow and /data, whose time goes to the
   full searches).  The translation unit of an instantiation chooses
   NEBC7_SHARED to match. */
constexpr int kShapeCompact = 0;
constexpr int kShapeOutlined = 1;

/* Resident CTAs per SM the compact refining kernel is compiled for (bounds
   its registers per thread; the draft-only kernels and the outlined shape
   are compiled for 4). */
#ifndef NEBC7_COMPACT_MIN_CTAS
#define NEBC7_COMPACT_MIN_CTAS 1
#endif

/* Persistent encode kernel over a launch's textures.  NORMAL compiles the
   refinement / full-search passes (run for textures whose preset asks for
   them); only that instantiation reserves the per-warp search state in
   shared memory.  kD: the kDenoise of every texture, or kAnyDenoise. */
template<int kD, bool NORMAL, int SHAPE>
__global__ void __launch_bounds__(kWarpsPerCta * 32, (SHAPE == kShapeOutlined || !NORMAL) ? 4 : NEBC7_COMPACT_MIN_CTAS)
	KEncode(Job job, LevelTables T0, LevelTables T1)
{
	extern __shared__ __align__(16) unsigned char encodeSmem[];
	const int lane = threadIdx.x & 31;
	const int warp = threadIdx.x >> 5;
	WarpState& st = reinterpret_cast<WarpState*>(encodeSmem)[warp];
	SearchState* ss = NORMAL ? reinterpret_cast<SearchState*>(encodeSmem + kWarpsPerCta * sizeof(WarpState)) + warp : nullptr;
	for (;;)
	{
		int k = 0;
		if (lane == 0)
			k = atomicAdd(job.counter, 1);
		k = __shfl_sync(kFull, k, 0);
		if (k >= job.total)
			break;
		EncodeQueued<kD, NORMAL>(st, ss, job, T0, T1, k, lane);
	}
}

/* Host-side launchers of KEncode.  Each instantiation is compiled in a
   translation unit of its own (encode_d<kD>_<passes>.cu), so they build in
   parallel; the C ABI layer only sees these declarations. */
template<int kD, bool NORMAL, int SHAPE>
cudaError_t LaunchEncodeKernel(int grid, cudaStream_t stream, const Job& job, const LevelTables& T0, const LevelTables& T1);

template<int kD, bool NORMAL, int SHAPE>
cudaError_t EncodeKernelOccupancy(int* ctasPerSm);

} // namespace nebc7
