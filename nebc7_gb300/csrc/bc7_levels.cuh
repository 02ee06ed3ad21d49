/*
 * BC7 block encoder for sm_103a -- per-channel candidate endpoint lists and
 * lower-bound estimates, warp-cooperative.
 *
 * ChannelLevels reproduces the reference's LevelsBuffer::
 * ComputeChannelLevelsReduced (src/SnippetLevelsBuffer.h:43-270), the nibble
 * variant of src/SnippetLevelsBufferHalf.h:43-223 and the single-best
 * variant (:148-188).  For one channel of one pixel subset it enumerates a
 * window of quantised endpoint pairs c, scores each by
 *   e(c) = sum_i D(x_i, c)^2   (D from the level tables),
 * keeps those with e < top, and returns the maxSize smallest keys
 * (e << 16 | c) in ascending order.  The reference collects all survivors
 * and radix-sorts them stably on e; since survivors are produced in
 * ascending c, that is the same as the smallest keys of the 32-bit key, which
 * is what the warp keeps here: lanes score 32 candidates at a time and a
 * bitonic merge folds them into a lane-resident sorted top-N.  Candidates are
 * visited in ascending c, so once the list is full a later candidate can only
 * enter with a strictly smaller error.
 *
 * The window arithmetic keeps the reference's 32-bit wrap-around behaviour
 * (its water can be negative for a later channel of a subset), and the
 * candidate set follows the chunking of its 16-wide AVX2 scan.
 */
#pragma once

#include "bc7_block.cuh"

namespace nebc7 {

struct ChanList
{
	int minErr;
	int count;
};

__device__ __forceinline__ int Wadd(int a, int b) { return int(unsigned(a) + unsigned(b)); }
__device__ __forceinline__ int Wsub(int a, int b) { return int(unsigned(a) - unsigned(b)); }
__device__ __forceinline__ unsigned Shr32(unsigned v, unsigned s) { return v >> (s & 31); }

/* Whether the scans read the reduced tables of 2- and 3-bit indices through
   the 8-bit difference tables (DiffBase) or in the reference's per-x
   layout.  The difference tables serve the full searches best; the compact
   default-preset kernel, whose time goes to the Mode6Index2 refinement,
   keeps the per-x layout (its translation unit sets 0). */
#ifndef NEBC7_REDUCED_BY_DIFF
#define NEBC7_REDUCED_BY_DIFF 1
#endif
constexpr bool kReducedByDiff = NEBC7_REDUCED_BY_DIFF != 0;

/* A reduced table's s-bit endpoint expanded to 8 bits by bit replication. */
__device__ __forceinline__ int ExpandTo8(int v, int s)
{
	return s >= 8 ? v : ((v << (8 - s)) | (v >> (2 * s - 8)));
}

/* The reduced tables of s-bit endpoints hold, for every x, the 8-bit
   table's entry at the expanded endpoints; the 8-bit byte tables of 2- and
   3-bit indices are stored by endpoint differences (DiffAt).  For
   candidate cc (endpoints cc >> s, cc & (2^s - 1)) the difference-table
   entry of channel value x is table[DiffBase(cc, s) - 513 x]: one lookup
   per term, as in the per-x layout, but in a region near the table's
   diagonal that every block shares, where the per-x rows of the distinct
   values of a channel lie far apart. */
__device__ __forceinline__ int DiffBase(int cc, int s)
{
	const int eH = ExpandTo8(cc >> s, s), eL = ExpandTo8(cc & ((1 << s) - 1), s);
	return (eH << 9) + eL + 255 * 513;
}

/* d with d*d < top (src/SnippetLevelsBuffer.h:78-88): truncated single
   precision square root, NaN (negative top) giving INT_MIN. */
template<int kD>
__device__ __forceinline__ int WindowRadius(int top)
{
	int d;
	if (top < 0)
		d = int(0x80000000u);
	else
		d = __float2int_rz(__fsqrt_rn(__int2float_rn(top)));
	const int sq = int(unsigned(d) * unsigned(d));   /* x86 imul wraps */
	d = Wsub(d, sq >= top ? 1 : 0);
	if (kD)
	{
		d = int(unsigned(d) << kD);
		d = Wadd(d, (1 << kD) - 1);
	}
	return d;
}

struct Window
{
	int LH, HL, HH;
};

/* src/SnippetLevelsBuffer.h:122-132 */
__device__ __forceinline__ Window MakeWindow(int L, int H, int d, int bits, int shift)
{
	const int tailmask = (1 << (8 - bits)) - 1;
	int LH = min(Wadd(L, d), 255);
	int HL = max(Wsub(H, d), 0);
	LH = min(Wadd(Wsub(H, H >> shift), tailmask), Wsub(LH, LH >> shift)) & ~tailmask;
	HL = max(Wsub(L, L >> shift), Wadd(Wsub(HL, HL >> shift), tailmask)) & ~tailmask;
	Window w;
	w.LH = LH >> (8 - shift);
	w.HL = HL >> (8 - shift);
	w.HH = 0x100 >> (8 - shift);
	return w;
}

/* Packed candidate index -> endpoint pair color (e0 | e1 << 8), honouring a
   channel whose oriented bounds run high to low (src/SnippetLevelsBuffer.h:230-268). */
__device__ __forceinline__ int DecodeColor(int c, int shift, bool reverse)
{
	if (reverse)
	{
		const int cL = (c >> shift) << (8 - shift);
		const int cH = (c & ((1 << shift) - 1)) << (8 - shift);
		return ((cH + (cH >> shift)) << 8) + cL + (cL >> shift);
	}
	if (shift != 8)
	{
		const int cH = (c >> shift) << (8 - shift);
		const int cL = (c & ((1 << shift) - 1)) << (8 - shift);
		return ((cH + (cH >> shift)) << 8) + cL + (cL >> shift);
	}
	return c;
}

/* Lane-resident sorted list of the N smallest keys (lane j holds the j-th). */
__device__ __forceinline__ unsigned BitonicSort32(unsigned v, int lane)
{
#pragma unroll
	for (int k = 2; k <= 32; k <<= 1)
	{
#pragma unroll
		for (int j = k >> 1; j > 0; j >>= 1)
		{
			const unsigned o = __shfl_xor_sync(kFull, v, j);
			const bool keepMin = ((lane & j) == 0) == ((lane & k) == 0);
			v = keepMin ? min(v, o) : max(v, o);
		}
	}
	return v;
}

__device__ __forceinline__ unsigned MergeTop(unsigned list, unsigned batch, int lane, int N)
{
	const unsigned s = BitonicSort32(batch, lane);
	const unsigned r = __shfl_sync(kFull, s, 31 - lane);
	unsigned m = min(list, r);
#pragma unroll
	for (int j = 16; j > 0; j >>= 1)
	{
		const unsigned o = __shfl_xor_sync(kFull, m, j);
		m = ((lane & j) == 0) ? min(m, o) : max(m, o);
	}
	return lane < N ? m : 0xFFFFFFFFu;
}

/* The distinct values of channel `offset` among the first `count` pixels,
   with their multiplicities, into uniq[] (value | count << 16); returns how
   many.  The scans sum a candidate's error once per distinct value (the
   integer sums, and so the saturated ones, are the same). */
__device__ __forceinline__ int UniqueValues(const Area& ar, int count, int offset, int* uniq, int lane)
{
	const int x = lane < count ? int(ar.px[lane & 15][offset]) : -1 - lane;
	const unsigned peers = __match_any_sync(kFull, x);
	const bool leader = lane < count && (__ffs(peers) - 1) == lane;
	const unsigned lm = __ballot_sync(kFull, leader);
	const int n = __popc(lm);
	if (leader)
		uniq[__popc(lm & ((1u << lane) - 1))] = x | (__popc(peers) << 16);
	/* zero entries (value 0, count 0) up to a multiple of 4, so that a scan
	   can read four at a time */
	if (lane >= n && lane < ((n + 3) & ~3))
		uniq[lane] = 0;
	__syncwarp();
	return n;
}

/* Sets node 0 (a zero-error candidate) of a list. */
__device__ __forceinline__ ChanList ZeroList(int2* nodes, int color, int lane)
{
	if (lane == 0)
		nodes[0] = make_int2(0, color);
	__syncwarp();
	return ChanList{ 0, 1 };
}

/* LevelsBuffer and LevelsBufferHalf: writes up to maxSize nodes (err, color). */
template<int kD, bool HALF>
__device__ __forceinline__ ChanList ChannelLevelsScan(int2* nodes, const Area& ar, const AreaInfo& ai, int offset, int weight,
	int water, int bits, int pbits, bool transparent, const uint8_t* table, bool byDiff, int maxSize, int* uniq, int lane)
{
	ChanList res{ MaxColorError<kD>() * 2, 0 };
	const int shift = bits + int(pbits >= 0 || HALF);
	const int count = transparent ? ai.active : ai.count;
	if (transparent && !count)
		return ZeroList(nodes, (pbits < 0) ? 0 : (pbits << (7 - bits)), lane);

	int top = (water + weight - 1) / weight;
	if (!top)
		return res;
	const int d = WindowRadius<kD>(top);

	const int L = int(int16_t(ai.minmax[2 * offset]));
	const int H = int(int16_t(ai.minmax[2 * offset + 1]));
	const bool reverse = (L != int(int16_t(ai.bounds[2 * offset])));

	if ((pbits < 0) || ((pbits >> 8) == (pbits & 1)))
	{
		if (L == H && ((((L >> shift) ^ L) & ((1 << (8 - shift)) - 1)) == 0))
		{
			if ((pbits < 0) || (((L >> (8 - shift)) & 1) == (pbits & 1)))
				return ZeroList(nodes, (H << 8) + L, lane);
		}
	}

	const Window win = MakeWindow(L, H, d, bits, shift);
	unsigned top16;
	if (HALF)
	{
		top = min(top, 15 * 15 * 16 + 1);
		top16 = unsigned(top);
	}
	else
	{
		if (top > 0xFFFF)
			top = 0xFFFF;
		top16 = unsigned(top) & 0xFFFF;
	}
	const bool topNeg = HALF && top < 0;   /* signed compare rejects everything */

	/* byte tables by (x, c); with 8-bit endpoints (shift 8) the byte table
	   goes by DiffAt and the half tables by HalfAt */
	const int rowSize = 1 << (2 * shift);
	const bool diff = shift == 8 || (kReducedByDiff && byDiff);
	const int nu = UniqueValues(ar, count, offset, uniq, lane);
	const bool pvar = HALF || pbits >= 0;
	const int pH = reverse ? (pbits & 1) : (pbits >> 8);
	const int pL = reverse ? (pbits >> 8) : (pbits & 1);

	/* list: the maxSize smallest keys so far, lane j the j-th; thr: its last
	   key (all ones until the list is full), which changes only on a merge.
	   The number of kept candidates matters only up to maxSize, which is the
	   number of filled list entries, and a list whose last key has error 0
	   means maxSize zero-error candidates were found. */
	unsigned list = 0xFFFFFFFFu;
	unsigned thr = 0xFFFFFFFFu;
	const int rowStep = pvar ? 2 : 1;
	/* hL - cH = LH for every row: when LH is below one chunk, only the first
	   chunk of a row can be on and a batch takes two rows (lanes 16..31 the
	   second); the candidate set and the kept keys are unchanged */
	const int W = pvar ? 32 : 16;
	const bool twoRows = win.LH < W;
	for (int iH0 = win.HL + (pvar ? pH : 0); iH0 < win.HH; iH0 += twoRows ? 2 * rowStep : rowStep)
	{
		/* candidates in batches of 32: two 16-candidate chunks per batch */
		for (int b = 0;; b++)
		{
			const int half = lane >> 4, j = lane & 15;
			const int iH = twoRows ? iH0 + half * rowStep : iH0;
			const int cH = iH << shift;
			const int hL = win.LH + cH;
			const int chunk = twoRows ? b : 2 * b + half;
			int c, cc;
			unsigned flags;
			if (pvar)
			{
				c = cH + 32 * chunk;
				cc = c + pL + 2 * j;
				flags = Shr32(~0u, unsigned(max(0, Wsub(c | 31, hL | 7))));
			}
			else
			{
				c = cH + 16 * chunk;
				cc = c + j;
				flags = Shr32(~0u, unsigned(max(0, Wsub(c | 15, hL | 7))) << 1);
			}
			const bool chunkOn = (iH < win.HH) && ((c == cH) || (c <= hL));
			const bool on = chunkOn && ((flags >> (2 * j)) & 1);
			if (!__any_sync(kFull, chunkOn))
				break;
			unsigned key = 0xFFFFFFFFu;
			if (on)
			{
				/* the per-x build reads the 8-bit table by DiffAt, as DiffBase with s = 8 */
				const int dbase = kReducedByDiff ? DiffBase(cc, shift) : 0;
				/* four distinct values per step, their table reads in flight
				   together (unsigned sums do not depend on the order) */
				auto term = [&](int e) {
					const int x = e & 0xFFFF;
					unsigned v;
					if (HALF)
						v = HalfAt(table, x, cc & 0xFF, cc >> 8);
					else if (diff)
						v = kReducedByDiff ? table[dbase - 513 * x] : DiffAt(table, x, cc & 0xFF, cc >> 8);
					else
						v = table[size_t(x) * rowSize + cc];
					return unsigned(e >> 16) * v * v;
				};
				unsigned s = 0;
				for (int u = 0; u < nu; u += 4)
				{
					const int4 e4 = *reinterpret_cast<const int4*>(uniq + u);
					s += (term(e4.x) + term(e4.y)) + (term(e4.z) + term(e4.w));
				}
				if (!HALF && s > 0xFFFF)
					s = 0xFFFF;
				const bool keep = HALF ? (!topNeg && int(s) < top) : (s < top16);
				if (keep)
					key = (s << 16) | unsigned(cc);
			}
			if (__any_sync(kFull, key < thr))
			{
				list = MergeTop(list, key < thr ? key : 0xFFFFFFFFu, lane, maxSize);
				thr = __shfl_sync(kFull, list, maxSize - 1);
			}
		}
		/* maxSize zero-error candidates found: later ones (larger c) cannot enter */
		if (thr < 0x10000u)
			break;
	}
	const int stored = __popc(__ballot_sync(kFull, list != 0xFFFFFFFFu));
	if (stored)
	{
		res.count = stored;
		const unsigned k0 = __shfl_sync(kFull, list, 0);
		res.minErr = int(k0 >> 16) * weight;
		if (lane < res.count)
			nodes[lane] = make_int2(int(list >> 16) * weight, DecodeColor(int(list & 0xFFFF), shift, reverse));
	}
	__syncwarp();
	return res;
}

/* Out-of-line copy of the scan for its many call sites; the Mode6Index2
   refinement (the common case of the default preset) inlines the scan. */
template<int kD, bool HALF>
__device__ NEBC7_SHARED ChanList ChannelLevels(int2* nodes, const Area& ar, const AreaInfo& ai, int offset, int weight, int water,
	int bits, int pbits, bool transparent, const uint8_t* table, bool byDiff, int maxSize, int* uniq, int lane)
{
	return ChannelLevelsScan<kD, HALF>(nodes, ar, ai, offset, weight, water, bits, pbits, transparent, table, byDiff, maxSize, uniq,
		lane);
}

/* Single best candidate over the narrower window of the alpha slot of modes
   4 and 5 (src/SnippetLevelsBuffer.h:148-188, 433-490). */
template<int kD>
__device__ NEBC7_SHARED ChanList ChannelLevelsSingle(int2* nodes, const Area& ar, const AreaInfo& ai, int offset, int weight, int water,
	int bits, bool transparent, const uint8_t* table, bool byDiff, int* uniq, int lane)
{
	ChanList res{ MaxColorError<kD>() * 2, 0 };
	const int shift = bits;
	const int count = transparent ? ai.active : ai.count;
	if (transparent && !count)
		return ZeroList(nodes, 0, lane);
	int top = (water + weight - 1) / weight;
	if (!top)
		return res;
	const int d = WindowRadius<kD>(top);
	const int L = int(int16_t(ai.minmax[2 * offset]));
	const int H = int(int16_t(ai.minmax[2 * offset + 1]));
	const bool reverse = (L != int(int16_t(ai.bounds[2 * offset])));
	if (L == H && ((((L >> shift) ^ L) & ((1 << (8 - shift)) - 1)) == 0))
		return ZeroList(nodes, (H << 8) + L, lane);
	const Window win = MakeWindow(L, H, d, bits, shift);
	if (top > 0xFFFF)
		top = 0xFFFF;
	const unsigned top16 = unsigned(top) & 0xFFFF;
	const int rowSize = 1 << (2 * shift);
	const bool diff = shift == 8 || (kReducedByDiff && byDiff);   /* DiffBase */
	const int nu = UniqueValues(ar, count, offset, uniq, lane);

	unsigned best = 0xFFFFFFFFu;
	/* two rows per batch when only a row's first chunk can be on */
	const bool twoRows = win.LH < 16;
	for (int iH0 = win.HL; iH0 < win.HH; iH0 += twoRows ? 2 : 1)
	{
		for (int b = 0;; b++)
		{
			const int half = lane >> 4, j = lane & 15;
			const int iH = twoRows ? iH0 + half : iH0;
			const int cH = iH << shift;
			const int hL = min(win.LH, iH) + cH;
			const int c = cH + 16 * (twoRows ? b : 2 * b + half);
			const int cc = c + j;
			const unsigned mask = Shr32(~0u, unsigned(max(0, Wsub(c | 15, hL | 7))) << 1);
			const bool chunkOn = (iH < win.HH) && ((c == cH) || (c <= hL));
			if (!__any_sync(kFull, chunkOn))
				break;
			if (chunkOn && ((mask >> (2 * j)) & 1))
			{
				const int dbase = kReducedByDiff ? DiffBase(cc, shift) : 0;
				auto term = [&](int e) {
					const int x = e & 0xFFFF;
					const unsigned v = diff ? (kReducedByDiff ? table[dbase - 513 * x] : DiffAt(table, x, cc & 0xFF, cc >> 8))
					                        : table[size_t(x) * rowSize + cc];
					return unsigned(e >> 16) * v * v;
				};
				unsigned s = 0;
				for (int u = 0; u < nu; u += 4)
				{
					const int4 e4 = *reinterpret_cast<const int4*>(uniq + u);
					s += (term(e4.x) + term(e4.y)) + (term(e4.z) + term(e4.w));
				}
				if (s > 0xFFFF)
					s = 0xFFFF;
				if (s < top16)
					best = min(best, (s << 16) | unsigned(cc));
			}
		}
	}
	best = __reduce_min_sync(kFull, best);
	if (best != 0xFFFFFFFFu)
	{
		const int e = int(best >> 16) * weight;
		res.minErr = e;
		res.count = 1;
		if (lane == 0)
			nodes[0] = make_int2(e, DecodeColor(int(best & 0xFFFF), shift, reverse));
	}
	__syncwarp();
	return res;
}

/* LevelsMinimum::EstimateChannelLevelsReduced (src/SnippetLevelsMinimum.h:117-311):
   the smallest e(c) over the window (or top), rows pruned by their cut-table
   lower bound.  The minimum does not depend on the visiting order, so rows
   are visited in order with the running best. */
template<int kD>
__device__ NEBC7_SHARED int EstimateChannelLevels(const Area& ar, const AreaInfo& ai, int offset, int weight, int water, int bits,
	bool transparent, const uint8_t* table, bool byDiff, const uint16_t* tower, int* uniq, int lane)
{
	const int shift = bits;
	const int count = transparent ? ai.active : ai.count;
	if (transparent && !count)
		return 0;
	int top = (water + weight - 1) / weight;
	if (!top)
		return 0;
	const int d = WindowRadius<kD>(top);
	const int L = int(int16_t(ai.minmax[2 * offset]));
	const int H = int(int16_t(ai.minmax[2 * offset + 1]));
	if (L == H)
		return 0;
	if (bits == 7 && H - L <= 5)
		return 0;
	if (bits == 8 && H - L <= 3)
		return 0;
	const Window win = MakeWindow(L, H, d, bits, shift);
	if (top > 0xFFFF)
		top = 0xFFFF;
	const int rowSize = 1 << (2 * bits);
	const bool diff = bits == 8 || (kReducedByDiff && byDiff);   /* DiffBase */
	const int towerSize = 1 << bits;
	const int nu = UniqueValues(ar, count, offset, uniq, lane);

	int best = top;
	for (int base = win.HL; base < win.HH; base += 32)
	{
		/* lane k holds the cut bound of row base + k */
		const int iHl = base + lane;
		unsigned rowLb = 0xFFFF;
		if (iHl < win.HH)
		{
			auto cut = [&](int e) { return unsigned(e >> 16) * tower[size_t(e & 0xFFFF) * towerSize + iHl]; };
			unsigned s = 0;
			for (int u = 0; u < nu; u += 4)
			{
				const int4 e4 = *reinterpret_cast<const int4*>(uniq + u);
				s += (cut(e4.x) + cut(e4.y)) + (cut(e4.z) + cut(e4.w));
			}
			rowLb = s > 0xFFFF ? 0xFFFF : s;
		}
		const int nrows = min(32, win.HH - base);
		for (int r = 0; r < nrows; r++)
		{
			const int lb = int(__shfl_sync(kFull, rowLb, r));
			if (lb >= best)
				continue;
			const int iH = base + r;
			const int cH = iH << shift;
			unsigned rowBest = 0xFFFF;
			for (int iL = cH, hL = min(win.LH, iH) + cH; iL <= hL; iL += 32)
			{
				/* cc = iL + lane stays in row iH (iL <= hL, iL - cH a multiple of 32) */
				const int cc = iL + lane;
				const int dbase = kReducedByDiff ? DiffBase(cc, bits) : 0;
				auto term = [&](int e) {
					const int x = e & 0xFFFF;
					const unsigned v = diff ? (kReducedByDiff ? table[dbase - 513 * x] : DiffAt(table, x, cc & 0xFF, cc >> 8))
					                        : table[size_t(x) * rowSize + cc];
					return unsigned(e >> 16) * v * v;
				};
				unsigned s = 0;
				for (int u = 0; u < nu; u += 4)
				{
					const int4 e4 = *reinterpret_cast<const int4*>(uniq + u);
					s += (term(e4.x) + term(e4.y)) + (term(e4.z) + term(e4.w));
				}
				if (s > 0xFFFF)
					s = 0xFFFF;
				rowBest = min(rowBest, s);
			}
			rowBest = __reduce_min_sync(kFull, rowBest);
			best = min(best, int(rowBest));
		}
	}
	return best * weight;
}

} // namespace nebc7
