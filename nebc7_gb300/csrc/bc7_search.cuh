/*
 * BC7 block encoder for sm_103a -- refinement and full searches (the
 * reference's "normal" and "slow" passes, ModeN::CompressBlock and
 * ModeN::CompressBlockFull).
 *
 * The exhaustive search over per-channel candidate lists (the reference's
 * TryVariants) visits combinations in a fixed nested order and keeps each
 * one whose error is strictly below the running best ("water"), skipping
 * combinations by comparing bounds (a sorted channel error plus the other
 * channels' minima, or a memoised error over a subset of channels) with the
 * water.  The warp keeps the outer loops uniform and in order, computes the
 * memoised subset-of-channel errors for a whole loop level at once (lane =
 * list entry, early exit at the water in force when the level starts, which
 * decides every later comparison the same way), evaluates the innermost
 * channel's candidates in parallel and then replays the innermost loop's
 * acceptances in order (ReplayInner), so that the result matches the
 * sequential search even where masked pixels make a bound exceed the error.
 */
#pragma once

#include "bc7_fast.cuh"
#include "bc7_levels.cuh"
#include "bc7_pca.cuh"

namespace nebc7 {

constexpr bool kHasNormalPasses = true;


constexpr int kBig = 0x7FFFFFFF;

struct __align__(16) SearchState
{
	int2 lists[4][4][32];    /* [p-bit variant][channel][entry] = (error, color) */
	int planes[3][256];      /* partial error planes of the combination search, [pixel][level] */
	int2 order[64];          /* full searches: (estimate, partition) */
	int est[64][3][3];       /* per partition, subset, channel (G, R, B) estimates */
	int lines[64][2];        /* per partition, estimates of subsets 2 and 3 */
	int uniq[16];            /* distinct channel values of the subset being scanned */
};

/* ---------------------------------------------------------------------- */
/* Partial error planes                                                   */
/*                                                                        */
/* For endpoints fixed on some channels, plane[i][k] holds the weighted   */
/* squared distances of pixel i to level k summed over those channels.    */
/* A candidate for one more channel then costs one channel per pixel and  */
/* level instead of all four; the sums are the same integers.             */
/* ---------------------------------------------------------------------- */

/* dst[i][k] = src[i][k] (0 without src) + w * q(x_i,c - v_k(col))^2 for the
   first np pixels of the area, L = 1 << IB levels. */
template<int kD, int IB>
__device__ __forceinline__ void PlaneAdd(int* dst, const int* src, const Area& ar, int np, int c, int col, int w, int lane)
{
	constexpr int L = 1 << IB;
	const int e0 = col & 0xFF, e1 = (col >> 8) & 0xFF;
	/* entry e = lane + 32 m has level e & (L - 1) = lane & (L - 1) */
	const int v = Interp(e0, e1, InterpWeights(IB)[lane & (L - 1)]);
	for (int e = lane; e < np * L; e += 32)
	{
		const int q = Q<kD>(int(ar.px[e >> IB][c]) - v);
		dst[e] = (src ? src[e] : 0) + w * q * q;
	}
	__syncwarp();
}

/* sum_i min_k (plane[i][k] + w * q(x_i,c - v_k(col))^2), stopping once the
   sum reaches `limit` (the same partial sums as the four-channel error). */
template<int kD, int IB>
__device__ __forceinline__ int PlaneError(const int* plane, const Area& ar, int np, int c, int col, int w, int limit)
{
	constexpr int L = 1 << IB;
	const int* wk = InterpWeights(IB);
	const int e0 = col & 0xFF, e1 = (col >> 8) & 0xFF;
	int v[L];
#pragma unroll
	for (int k = 0; k < L; k++)
		v[k] = Interp(e0, e1, wk[k]);
	int sum = 0;
	for (int i = 0; i < np; i++)
	{
		const int x = ar.px[i][c];
		const int4* row = reinterpret_cast<const int4*>(plane + i * L);
		int best = kBig;
#pragma unroll
		for (int k4 = 0; k4 < L / 4; k4++)
		{
			const int4 pv = row[k4];
			const int q0 = Q<kD>(x - v[4 * k4]), q1 = Q<kD>(x - v[4 * k4 + 1]);
			const int q2 = Q<kD>(x - v[4 * k4 + 2]), q3 = Q<kD>(x - v[4 * k4 + 3]);
			best = min(best, min(min(pv.x + w * q0 * q0, pv.y + w * q1 * q1), min(pv.z + w * q2 * q2, pv.w + w * q3 * q3)));
		}
		sum += best;
		if (!(limit > sum))
			break;
	}
	return sum;
}

/* ---------------------------------------------------------------------- */
/* Errors over an area, with early exit at `water` (only used to reject)   */
/* ---------------------------------------------------------------------- */

template<int kD, int BITS>
__device__ NEBC7_PASS int AreaError(const Area& ar, int active, Ep ep, const int w[4], int water)
{
	LevelSet<BITS> Lv;
	Lv.Init(ep);
	int sum = 0;
	for (int i = 0; i < active; i++)
	{
		const int p0 = ar.px[i][0], p1 = ar.px[i][1], p2 = ar.px[i][2], p3 = ar.px[i][3];
		int best = kBig;
#pragma unroll
		for (int k = 0; k < (1 << BITS); k++)
		{
			const int q0 = Q<kD>(p0 - Lv.v[k][0]), q1 = Q<kD>(p1 - Lv.v[k][1]);
			const int q2 = Q<kD>(p2 - Lv.v[k][2]), q3 = Q<kD>(p3 - Lv.v[k][3]);
			best = min(best, w[0] * q0 * q0 + w[1] * q1 * q1 + w[2] * q2 * q2 + w[3] * q3 * q3);
		}
		sum += best;
		if (!(water > sum))
			break;
	}
	return sum;
}

/* Mode 4/5 error on Area1 (see RotErrorExact) with early exit. */
template<int kD, int CB, int AB, bool MODE4>
__device__ NEBC7_PASS int RotErrorW(const Area& ar, const AreaInfo& ai, Ep epImg, int rotation, const int w[4], int water)
{
	const int a = RotChannel(rotation);
	LevelSet<CB> LC;
	LevelSet<AB> LA;
	LC.Init(epImg);
	LA.Init(epImg);
	int sum = 0;
	const int n = MODE4 ? ai.active : 16;
	for (int i = 0; i < n; i++)
	{
		int px[4], mk[4];
#pragma unroll
		for (int c = 0; c < 4; c++)
		{
			px[c] = ar.px[i][c];
			mk[c] = ar.mk[i][c];
		}
		int bestc = kBig;
#pragma unroll
		for (int k = 0; k < (1 << CB); k++)
		{
			int e = 0;
#pragma unroll
			for (int c = 0; c < 4; c++)
			{
				const int q = Q<kD>(px[c] - LC.v[k][c]);
				e += (c == a) ? 0 : w[c] * ((q * q) & mk[c]);
			}
			bestc = min(bestc, e);
		}
		int besta = kBig;
#pragma unroll
		for (int k = 0; k < (1 << AB); k++)
		{
			int e = 0;
#pragma unroll
			for (int c = 0; c < 4; c++)
			{
				const int q = Q<kD>(px[c] - LA.v[k][c]);
				e += (c == a) ? w[c] * ((q * q) & mk[c]) : 0;
			}
			besta = min(besta, e);
		}
		sum += besta;
		sum += bestc;
		if (!(water > sum))
			return sum;
	}
	if (MODE4 && ai.active < 16)
	{
		const int m = min(EpGet(epImg, 0), EpGet(epImg, 1));
		const int q = Q<kD>(m);
		sum += q * q * (w[0] * (16 - ai.active));
	}
	return sum;
}

__device__ __forceinline__ Ep Ep2(int c0, int col0, int c1, int col1)
{
	return EpSetCh(EpSetCh(0, c0, col0), c1, col1);
}

/* The innermost loop of a combination search, replayed in the reference's
   order.  Lane j holds candidate j of the innermost (sorted) list: `brk` is
   its sorted bound (the loop ends at the first lane with brk >= water),
   `skip` its memoised bound (the lane is passed over when skip >= water) and
   `err` its error, computed with an early exit at the water in force when
   the loop started (exact whenever below it).  A lane is accepted when, at
   the running water, it is the first later lane with all three below the
   water; the water then drops to its error.  With arbitrary pixel masks the
   bounds are not always lower bounds of the error, so the order matters.
   Returns the last accepted lane or -1. */
__device__ __forceinline__ int ReplayInner(bool valid, int brk, int skip, int err, int& water, int lane)
{
	int taken = -1;
	for (;;)
	{
		const unsigned m = __ballot_sync(kFull, valid && lane > taken && brk < water && skip < water && err < water);
		if (!m)
			break;
		taken = __ffs(m) - 1;
		water = __shfl_sync(kFull, err, taken);
	}
	return taken;
}

/* ---------------------------------------------------------------------- */
/* Modes 0-3: three channels G, R, B (src/Bc7CoreMode0.cpp:242-415)        */
/* ---------------------------------------------------------------------- */

template<int kD, int IB>
__device__ NEBC7_SHARED int TryVariants3(const Area& ar, const AreaInfo& ai, const Params& P, const int2* L1, ChanList c1,
	const int2* L2, ChanList c2, const int2* L3, ChanList c3, Ep& best, int water, int* planes, int lane)
{
	const int min1 = c1.minErr, min2 = c2.minErr, min3 = c3.minErr;
	if (min1 + min2 + min3 >= water)
		return water;
	const int n2 = c2.count, n3 = c3.count, np = ai.active;
	int* pG = planes;
	int* pGR = planes + 256;
	const int col2l = lane < n2 ? L2[lane].y : 0;
	const int col3 = lane < n3 ? L3[lane].y : 0;
	const int e3base = lane < n3 ? L3[lane].x : kBig;
	for (int i1 = 0; i1 < c1.count; i1++)
	{
		const int e1 = L1[i1].x;
		if (e1 + min2 + min3 >= water)
			break;
		const int col1 = L1[i1].y;
		/* memoised G+B errors (memGB) and G+R pair errors, one list entry per lane */
		PlaneAdd<kD, IB>(pG, nullptr, ar, np, 1, col1, P.wG, lane);
		int memGB = kBig, pairGR = kBig;
		if (lane < n3)
			memGB = PlaneError<kD, IB>(pG, ar, np, 3, col3, P.wB, water - min2);
		if (lane < n2)
			pairGR = PlaneError<kD, IB>(pG, ar, np, 2, col2l, P.wR, water - min3);
		for (int i2 = 0; i2 < n2; i2++)
		{
			const int e2s = L2[i2].x + e1;
			if (e2s + min3 >= water)
				break;
			const int col2 = L2[i2].y;
			const int e2 = __shfl_sync(kFull, pairGR, i2);
			if (e2 + min3 >= water)
				continue;
			const bool valid = lane < n3;
			const int brk = valid ? e3base + e2 : kBig;
			const int skip = valid ? memGB + min2 : kBig;
			const bool eval = valid && brk < water && skip < water;
			/* no lane evaluates: the replay accepts nothing, the plane is not needed */
			if (!__any_sync(kFull, eval))
				continue;
			PlaneAdd<kD, IB>(pGR, pG, ar, np, 2, col2, P.wR, lane);
			int err = kBig;
			if (eval)
				err = PlaneError<kD, IB>(pGR, ar, np, 3, col3, P.wB, water);
			const int jl = ReplayInner(valid, brk, skip, err, water, lane);
			if (jl >= 0)
				best = EpSetCh(Ep2(1, col1, 2, col2), 3, __shfl_sync(kFull, col3, jl));
		}
	}
	return water;
}

struct Spec3
{
	int bits;               /* candidate list bits */
	const uint8_t* table;   /* by differences (DiffBase) unless it is the shared-p-bit table */
	bool byDiff;
	int estBits;
	const uint16_t* estTower;
};

template<int MODE>
__device__ __forceinline__ Spec3 GetSpec3(const LevelTables& T)
{
	/* mode 1's shared p-bit table marks endpoint pairs of different parity
	   (0xFF), which its estimates read: it stays in the per-x layout */
	if (MODE == 0)
		return Spec3{ 4, kReducedByDiff ? T.d3v8 : T.d3v5, kReducedByDiff, 5, T.c3v5 };
	if (MODE == 1)
		return Spec3{ 6, T.d3v7s, false, 7, T.c3v7s };
	if (MODE == 2)
		return Spec3{ 5, kReducedByDiff ? T.d2v8 : T.d2v5, kReducedByDiff, 5, T.c2v5 };
	return Spec3{ 7, T.d2v8, true, 8, T.c2v8 };
}

template<int MODE>
__device__ __forceinline__ int NumVariants3() { return MODE == 2 ? 1 : (MODE == 1 ? 2 : 4); }

__device__ __forceinline__ int Pbits(int mode, int v)
{
	if (mode == 2)
		return -1;
	const int pb[4] = { 0x0101, 0, 1, 1 << 8 };
	return pb[v];
}

/* Subset::InitLevels (src/Bc7CoreMode0.cpp:249-268) for variant v. */
template<int kD, int MODE>
__device__ NEBC7_PASS bool InitLevels3(SearchState& ss, int v, const Area& ar, const AreaInfo& ai, const Params& P, const Spec3& sp,
	int water, const int est[3], ChanList cl[3], int lane)
{
	const int pb = Pbits(MODE, v);
	cl[0] = ChannelLevels<kD, false>(ss.lists[v][0], ar, ai, 1, P.wG, water - est[1] - est[2], sp.bits, pb, false, sp.table, sp.byDiff, 32,
		ss.uniq, lane);
	const int min1 = cl[0].minErr;
	if (min1 >= water)
		return false;
	cl[1] = ChannelLevels<kD, false>(ss.lists[v][1], ar, ai, 2, P.wR, water - min1 - est[2], sp.bits, pb, false, sp.table, sp.byDiff, 32,
		ss.uniq, lane);
	const int min2 = cl[1].minErr;
	if (min1 + min2 >= water)
		return false;
	cl[2] = ChannelLevels<kD, false>(ss.lists[v][2], ar, ai, 3, P.wB, water - min1 - min2, sp.bits, pb, false, sp.table, sp.byDiff, 32,
		ss.uniq, lane);
	return min1 + min2 + cl[2].minErr < water;
}

/* Subsets (src/Bc7CoreMode0.cpp:366-415): all variants' lists start from
   the same water, then the variants are searched in order. */
template<int kD, int MODE>
__device__ NEBC7_PASS int SearchSubset3(SearchState& ss, const Area& ar, const AreaInfo& ai, const Params& P, const LevelTables& T,
	int water, const int est[3], Ep& best, bool& any, int lane)
{
	constexpr int IB = (MODE == 0 || MODE == 1) ? 3 : 2;
	const Spec3 sp = GetSpec3<MODE>(T);
	ChanList cl[4][3];
	bool valid[4];
	any = false;
	for (int v = 0; v < NumVariants3<MODE>(); v++)
	{
		valid[v] = InitLevels3<kD, MODE>(ss, v, ar, ai, P, sp, water, est, cl[v], lane);
		any |= valid[v];
	}
	for (int v = 0; v < NumVariants3<MODE>(); v++)
		if (valid[v])
			water = TryVariants3<kD, IB>(ar, ai, P, ss.lists[v][0], cl[v][0], ss.lists[v][1], cl[v][1], ss.lists[v][2], cl[v][2],
				best, water, &ss.planes[0][0], lane);
	return water;
}

template<int kD>
__device__ NEBC7_PASS AreaInfo BuildSubset(WarpState& st, const CellRegs& R, const Params& P, Area& ar, int ns, int p, int s, int lane)
{
	const uint32_t part = ns == 3 ? c_part3[p] : c_part2[p];
	const uint32_t member = Member(part, s);
	const int anchor = Anchor(ns, p, s);
	AreaInfo ai = AreaStats(st, R, P, member);
	ai.zero = anchor;
	BuildAreaList(ar, st, R, member, anchor, lane);
	return ai;
}

/* ModeN::CompressBlock for modes 0-3 (src/Bc7CoreMode0.cpp:417-498). */
template<int kD, int MODE>
__device__ NEBC7_PASS void RefineOpaque(WarpState& st, SearchState& ss, CellRegs& R, const Params& P, const LevelTables& T, int lane)
{
	constexpr int NS = (MODE == 0 || MODE == 2) ? 3 : 2;
	constexpr int IB = (MODE == 0 || MODE == 1) ? 3 : 2;
	const int p = R.bestParam;
	Ep mc[3] = { R.best[0], R.best[1], R.best[2] };
	const int est[3] = { 0, 0, 0 };
	const int wGRB[4] = { 0, P.wG, P.wR, P.wB };
	int error = R.opaqueAlphaError;
	if (error < R.errTotal)
	{
		for (int s = 0; s < NS; s++)
		{
			const AreaInfo ai = BuildSubset<kD>(st, R, P, st.sub[0], NS, p, s, lane);
			const int water = AreaError<kD, IB>(st.sub[0], ai.active, mc[s], wGRB, MaxColorError<kD>());
			if (water)
			{
				bool any;
				Ep b = mc[s];
				const int w2 = SearchSubset3<kD, MODE>(ss, st.sub[0], ai, P, T, water, est, b, any, lane);
				if (any)
				{
					error += w2;
					mc[s] = b;
				}
				else
					error += water;
			}
		}
		if (R.errTotal > error)
		{
			R.errTotal = error;
			R.best[0] = mc[0];
			R.best[1] = mc[1];
			if (NS == 3)
				R.best[2] = mc[2];
		}
	}
}

/* EstimateLevels of modes 0-3 (src/Bc7CoreMode0.cpp:500-530). */
template<int kD>
__device__ NEBC7_PASS int EstimateLevels3(SearchState& ss, const Area& ar, const AreaInfo& ai, const Params& P, const Spec3& sp, int water,
	int est[4], int lane)
{
	int error = 0;
	if (error < water)
	{
		const int l1 = EstimateChannelLevels<kD>(ar, ai, 1, P.wG, water - error, sp.estBits, false, sp.table, sp.byDiff, sp.estTower, ss.uniq, lane);
		est[1] = l1;
		error += l1;
		if (error < water)
		{
			const int l2 = EstimateChannelLevels<kD>(ar, ai, 2, P.wR, water - error, sp.estBits, false, sp.table, sp.byDiff, sp.estTower, ss.uniq, lane);
			est[2] = l2;
			error += l2;
			if (error < water)
			{
				const int l3 = EstimateChannelLevels<kD>(ar, ai, 3, P.wB, water - error, sp.estBits, false, sp.table, sp.byDiff, sp.estTower, ss.uniq, lane);
				est[3] = l3;
				error += l3;
				if (error < water)
					return error;
			}
		}
	}
	return water;
}

__device__ __forceinline__ void StableSortOrder(int2* order, int n, int lane)
{
	/* stable sort by unsigned error (src/Bc7Core.cpp:564 radix_sort_partitions):
	   rank = number of entries that must precede */
	int2 mine[2];
	int rank[2];
	for (int h = 0; h < 2; h++)
	{
		const int i = lane + 32 * h;
		rank[h] = -1;
		if (i < n)
		{
			mine[h] = order[i];
			int r = 0;
			for (int k = 0; k < n; k++)
			{
				const unsigned ek = unsigned(order[k].x), ei = unsigned(mine[h].x);
				r += (ek < ei) || (ek == ei && k < i);
			}
			rank[h] = r;
		}
	}
	__syncwarp();
	for (int h = 0; h < 2; h++)
		if (rank[h] >= 0)
			order[rank[h]] = mine[h];
	__syncwarp();
}

/* Full searches of modes 0 and 2 (src/Bc7CoreMode0.cpp:532-642,
   src/Bc7CoreMode2.cpp:456-566). */
template<int kD, int MODE>
__device__ NEBC7_PASS void FullThreeSubsets(WarpState& st, SearchState& ss, CellRegs& R, const Params& P, const LevelTables& T, int lane)
{
	constexpr int NP = MODE == 0 ? 16 : 64;
	const Spec3 sp = GetSpec3<MODE>(T);
	const int step = R.denoiseStep;
	int count = 0;
	for (int p = 0; p < NP; p++)
	{
		if (R.personalMode == MODE && R.personalParam == p)
			continue;
		int e[3][4];
		const AreaInfo a1 = BuildSubset<kD>(st, R, P, st.sub[0], 3, p, 0, lane);
		const int water1 = R.errTotal - step - R.opaqueAlphaError;
		const int line1 = EstimateLevels3<kD>(ss, st.sub[0], a1, P, sp, water1, e[0], lane);
		if (line1 < water1)
		{
			const AreaInfo a2 = BuildSubset<kD>(st, R, P, st.sub[0], 3, p, 1, lane);
			const int water2 = water1 - line1;
			const int line2 = EstimateLevels3<kD>(ss, st.sub[0], a2, P, sp, water2, e[1], lane);
			if (line2 < water2)
			{
				const AreaInfo a3 = BuildSubset<kD>(st, R, P, st.sub[0], 3, p, 2, lane);
				const int water3 = water2 - line2;
				const int line3 = EstimateLevels3<kD>(ss, st.sub[0], a3, P, sp, water3, e[2], lane);
				if (line3 < water3)
				{
					if (lane == 0)
					{
						ss.lines[p][0] = line2;
						ss.lines[p][1] = line3;
						for (int s = 0; s < 3; s++)
							for (int c = 1; c < 4; c++)
								ss.est[p][s][c - 1] = e[s][c];
						ss.order[count] = make_int2(R.opaqueAlphaError + line1 + line2 + line3 + step, p);
					}
					count++;
				}
			}
		}
		__syncwarp();
	}
	__syncwarp();
	StableSortOrder(ss.order, count, lane);

	for (int i = 0; i < count; i++)
	{
		const int2 o = ss.order[i];
		if (o.x < R.errTotal)
		{
			const int p = o.y;
			Ep mc[3] = { 0, 0, 0 };
			const int line3 = ss.lines[p][1];
			int e1[3] = { ss.est[p][0][0], ss.est[p][0][1], ss.est[p][0][2] };
			const AreaInfo a1 = BuildSubset<kD>(st, R, P, st.sub[0], 3, p, 0, lane);
			const int water1 = R.errTotal - step - R.opaqueAlphaError - ss.lines[p][0] - line3;
			bool any;
			int error = SearchSubset3<kD, MODE>(ss, st.sub[0], a1, P, T, water1, e1, mc[0], any, lane);
			if (!any)
				continue;
			if (error < water1)
			{
				error += R.opaqueAlphaError;
				int e2[3] = { ss.est[p][1][0], ss.est[p][1][1], ss.est[p][1][2] };
				const AreaInfo a2 = BuildSubset<kD>(st, R, P, st.sub[0], 3, p, 1, lane);
				const int water2 = R.errTotal - step - error - line3;
				const int r2 = SearchSubset3<kD, MODE>(ss, st.sub[0], a2, P, T, water2, e2, mc[1], any, lane);
				if (!any)
					continue;
				error += r2;
				if (error < R.errTotal - step - line3)
				{
					int e3[3] = { ss.est[p][2][0], ss.est[p][2][1], ss.est[p][2][2] };
					const AreaInfo a3 = BuildSubset<kD>(st, R, P, st.sub[0], 3, p, 2, lane);
					const int water3 = R.errTotal - step - error;
					const int r3 = SearchSubset3<kD, MODE>(ss, st.sub[0], a3, P, T, water3, e3, mc[2], any, lane);
					if (!any)
						continue;
					error += r3;
					if (R.errTotal > error + step)
					{
						R.errTotal = error;
						R.best[0] = mc[0];
						R.best[1] = mc[1];
						R.best[2] = mc[2];
						R.bestParam = p;
						R.bestMode = MODE;
						if (error <= R.opaqueAlphaError)
							return;
					}
				}
			}
		}
	}
}

/* The partition search of modes 1 and 3 from its estimates (the second
   loop of src/Bc7CoreMode1.cpp:473-571, src/Bc7CoreMode3.cpp:471-569):
   partition p with the principal-axis bounds line1, line2 (0 without
   OPTION_PCA).  Returns true when the search ends the full pass. */
template<int kD, int MODE>
__device__ __forceinline__ bool TwoSubsetsPartition(WarpState& st, SearchState& ss, CellRegs& R, const Params& P, const Spec3& sp,
	const LevelTables& T, int p, int line1, int line2, int lane)
{
	const int step = R.denoiseStep;
	Ep mc[2] = { 0, 0 };
	int e1[4], e2[4];
	const AreaInfo a1 = BuildSubset<kD>(st, R, P, st.sub[0], 2, p, 0, lane);
	const AreaInfo a2 = BuildSubset<kD>(st, R, P, st.sub[1], 2, p, 1, lane);
	int w1 = R.errTotal - step - R.opaqueAlphaError - line2;
	line1 = max(line1, EstimateLevels3<kD>(ss, st.sub[0], a1, P, sp, w1, e1, lane));
	if (line1 < w1)
	{
		int w2 = w1 - line1;
		line2 = max(line2, EstimateLevels3<kD>(ss, st.sub[1], a2, P, sp, w2, e2, lane));
		if (line2 < w2)
		{
			w1 = R.errTotal - step - R.opaqueAlphaError - line2;
			const int est1[3] = { e1[1], e1[2], e1[3] };
			bool any;
			int error = SearchSubset3<kD, MODE>(ss, st.sub[0], a1, P, T, w1, est1, mc[0], any, lane);
			if (any && error < w1)
			{
				error += R.opaqueAlphaError;
				w2 = R.errTotal - step - error;
				const int est2[3] = { e2[1], e2[2], e2[3] };
				const int r2 = SearchSubset3<kD, MODE>(ss, st.sub[1], a2, P, T, w2, est2, mc[1], any, lane);
				if (any)
				{
					error += r2;
					if (R.errTotal > error + step)
					{
						R.errTotal = error;
						R.best[0] = mc[0];
						R.best[1] = mc[1];
						R.bestParam = p;
						R.bestMode = MODE;
						if (error <= R.opaqueAlphaError)
							return true;
					}
				}
			}
		}
	}
	return false;
}

/* Full searches of modes 1 and 3 (src/Bc7CoreMode1.cpp:473-571,
   src/Bc7CoreMode3.cpp:471-569).  Without OPTION_PCA every partition's
   bound is zero, so every partition enters with estimate OA + step and the
   stable sort keeps index order; with it, the partitions are estimated and
   sorted first (AreaGetBestPca3, src/Bc7Core.cpp:494).  Without OPTION_PCA
   the search may resume at partition `from` (the partitions before it
   searched already, R as they left it). */
template<int kD, int MODE>
__device__ NEBC7_PASS void FullTwoSubsets(WarpState& st, SearchState& ss, CellRegs& R, const Params& P, const LevelTables& T, int lane,
	int from = 0)
{
	const Spec3 sp = GetSpec3<MODE>(T);
	const int step = R.denoiseStep;
	if (!P.pca)
	{
		for (int p = from; p < 64; p++)
		{
			if (R.personalMode == MODE && R.personalParam == p)
				continue;
			if (!(0 < R.errTotal - step - R.opaqueAlphaError))
				continue;
			if (!(R.opaqueAlphaError + step < R.errTotal))
				continue;
			if (TwoSubsetsPartition<kD, MODE>(st, ss, R, P, sp, T, p, 0, 0, lane))
				return;
		}
		return;
	}
	int count = 0;
	for (int p = 0; p < 64; p++)
	{
		if (R.personalMode == MODE && R.personalParam == p)
			continue;
		const AreaInfo a1 = BuildSubset<kD>(st, R, P, st.sub[0], 2, p, 0, lane);
		const int water1 = R.errTotal - step - R.opaqueAlphaError;
		const int line1 = PcaBound<kD>(st.sub[0], a1, P, 3, lane);
		if (line1 < water1)
		{
			const AreaInfo a2 = BuildSubset<kD>(st, R, P, st.sub[1], 2, p, 1, lane);
			const int line2 = PcaBound<kD>(st.sub[1], a2, P, 3, lane);
			if (line2 < water1 - line1)
			{
				if (lane == 0)
				{
					ss.lines[p][0] = line1;
					ss.lines[p][1] = line2;
					ss.order[count] = make_int2(R.opaqueAlphaError + line1 + line2 + step, p);
				}
				count++;
			}
		}
		__syncwarp();
	}
	__syncwarp();
	StableSortOrder(ss.order, count, lane);
	for (int i = 0; i < count; i++)
	{
		const int2 o = ss.order[i];
		if (o.x < R.errTotal && TwoSubsetsPartition<kD, MODE>(st, ss, R, P, sp, T, o.y, ss.lines[o.y][0], ss.lines[o.y][1], lane))
			return;
	}
}

/* ---------------------------------------------------------------------- */
/* Modes 6, 6Index2, 7: four channels with the transparent-alpha term       */
/* ---------------------------------------------------------------------- */

template<int kD, int IB, bool T4>
__device__ __forceinline__ int TryVariants4Body(const Area& ar, const AreaInfo& ai, const Params& P, const LevelTables& T,
	const int2* const* Ls, const ChanList* cl, Ep& best, int water, int* planes, int lane)
{
	const int min0 = cl[0].minErr, min1 = cl[1].minErr, min2 = cl[2].minErr, min3 = cl[3].minErr;
	if (min0 + min1 + min2 + min3 >= water)
		return water;
	const int n1 = cl[1].count, n2 = cl[2].count, n3 = cl[3].count, np = ai.active;
	const bool opq = ai.opaque;
	const int2* L0 = Ls[0];
	const int2* L1 = Ls[1];
	const int2* L2 = Ls[2];
	const int2* L3 = Ls[3];
	/* an opaque area has alpha 255 and the alpha list holds 0xFFFF only, so the
	   alpha plane is zero and the A-less weights of the reference's opaque
	   branch give the same sums as the planes below */
	int* pA = planes;
	int* pAG = planes + 256;
	int* pAGR = planes + 512;
	const int col1l = lane < n1 ? L1[lane].y : 0;
	const int col2l = lane < n2 ? L2[lane].y : 0;
	const int col3 = lane < n3 ? L3[lane].y : 0;
	const int e3base = lane < n3 ? L3[lane].x : kBig;
	for (int i0 = 0; i0 < cl[0].count; i0++)
	{
		const int e0 = L0[i0].x;
		if (e0 + min1 + min2 + min3 >= water)
			break;
		const int c0 = L0[i0].y;
		const int ea = T4 ? TransparentError4(T, P, ai.count, ai.active, c0) : TransparentError2(T, P, ai.count, ai.active, c0);
		PlaneAdd<kD, IB>(pA, nullptr, ar, np, 0, c0, P.wA, lane);
		int memAR = kBig, pairAG = kBig;
		if (!opq)
		{
			if (lane < n2)
				memAR = PlaneError<kD, IB>(pA, ar, np, 2, col2l, P.wR, water - ea - min1 - min3) + ea;
			if (lane < n1)
				pairAG = PlaneError<kD, IB>(pA, ar, np, 1, col1l, P.wG, water - ea - min2 - min3) + ea;
		}
		for (int i1 = 0; i1 < n1; i1++)
		{
			int e1 = L1[i1].x + e0;
			if (e1 + min2 + min3 >= water)
				break;
			const int c1 = L1[i1].y;
			if (!opq)
			{
				e1 = __shfl_sync(kFull, pairAG, i1);
				if (e1 + min2 + min3 >= water)
					continue;
			}
			PlaneAdd<kD, IB>(pAG, pA, ar, np, 1, c1, P.wG, lane);
			const Ep base01 = Ep2(0, c0, 1, c1);
			int memAGB = kBig, pairAGR = kBig;
			if (lane < n3)
				memAGB = PlaneError<kD, IB>(pAG, ar, np, 3, col3, P.wB, water - ea - min2) + ea;
			if (lane < n2)
				pairAGR = PlaneError<kD, IB>(pAG, ar, np, 2, col2l, P.wR, water - ea - min3) + ea;
			for (int i2 = 0; i2 < n2; i2++)
			{
				const int e2s = L2[i2].x + e1;
				if (e2s + min3 >= water)
					break;
				const int c2 = L2[i2].y;
				if (!opq)
				{
					const int ear = __shfl_sync(kFull, memAR, i2);
					if (ear + min1 + min3 >= water)
						continue;
				}
				const int e2 = __shfl_sync(kFull, pairAGR, i2);
				if (e2 + min3 >= water)
					continue;
				const bool valid = lane < n3;
				const int brk = valid ? e3base + e2 : kBig;
				const int skip = valid ? memAGB + min2 : kBig;
				const bool eval = valid && brk < water && skip < water;
				/* no lane evaluates: the replay accepts nothing, the plane is not needed */
				if (!__any_sync(kFull, eval))
					continue;
				PlaneAdd<kD, IB>(pAGR, pAG, ar, np, 2, c2, P.wR, lane);
				const Ep base012 = EpSetCh(base01, 2, c2);
				int err = kBig;
				if (eval)
					err = PlaneError<kD, IB>(pAGR, ar, np, 3, col3, P.wB, water - ea) + ea;
				const int jl = ReplayInner(valid, brk, skip, err, water, lane);
				if (jl >= 0)
					best = EpSetCh(base012, 3, __shfl_sync(kFull, col3, jl));
			}
		}
	}
	return water;
}

/* Out-of-line copy for modes 6 and 7; the Mode6Index2 refinement (the
   common case of the default preset) inlines the body. */
template<int kD, int IB, bool T4>
__device__ NEBC7_SHARED int TryVariants4(const Area& ar, const AreaInfo& ai, const Params& P, const LevelTables& T, const int2* const* Ls,
	const ChanList* cl, Ep& best, int water, int* planes, int lane)
{
	return TryVariants4Body<kD, IB, T4>(ar, ai, P, T, Ls, cl, best, water, planes, lane);
}

/* Subset::InitLevels of modes 6 / 6Index2 / 7 (src/Bc7CoreMode6.cpp:1130-1161,
   src/Bc7CoreMode7.cpp:237-268). */
template<int kD, int MODE>
__device__ NEBC7_PASS bool InitLevels4(SearchState& ss, int v, int pbits, const Area& ar, const AreaInfo& ai, const Params& P,
	const LevelTables& T, int water, const int est[4], ChanList cl[4], int lane)
{
	const int wts[4] = { P.wA, P.wG, P.wR, P.wB };
	int used = 0;
	for (int c = 0; c < 4; c++)
	{
		int rest = 0;
		for (int k = c + 1; k < 4; k++)
			rest += est[k];
		if (c == 0 && ai.opaque)
		{
			cl[0] = ZeroList(ss.lists[v][0], 0xFFFF, lane);
		}
		else if (MODE == 6)
		{
			cl[c] = ChannelLevels<kD, true>(ss.lists[v][c], ar, ai, c, wts[c], water - used - rest, 7, pbits, c != 0, T.d4h, true, 20, ss.uniq,
				lane);
		}
		else if (MODE == 9)
		{
			cl[c] = ChannelLevelsScan<kD, true>(ss.lists[v][c], ar, ai, c, wts[c], water - used - rest, 7, pbits, c != 0, T.d2h, true, 20,
				ss.uniq, lane);
		}
		else
		{
			cl[c] = ChannelLevels<kD, false>(ss.lists[v][c], ar, ai, c, wts[c], water - used - rest, 5, pbits, c != 0, kReducedByDiff ? T.d2v8 : T.d2v6,
				kReducedByDiff, 20,
				ss.uniq, lane);
		}
		used += cl[c].minErr;
		if (used >= water)
			return false;
	}
	return true;
}

template<int kD, int MODE>
__device__ int TryV4(SearchState& ss, int v, const Area& ar, const AreaInfo& ai, const Params& P, const LevelTables& T,
	const ChanList cl[4], Ep& best, int water, int lane)
{
	const int2* Ls[4] = { ss.lists[v][0], ss.lists[v][1], ss.lists[v][2], ss.lists[v][3] };
	if (MODE == 6)
		return TryVariants4<kD, 4, true>(ar, ai, P, T, Ls, cl, best, water, &ss.planes[0][0], lane);
	if (MODE == 9)
		return TryVariants4Body<kD, 2, false>(ar, ai, P, T, Ls, cl, best, water, &ss.planes[0][0], lane);
	return TryVariants4<kD, 2, false>(ar, ai, P, T, Ls, cl, best, water, &ss.planes[0][0], lane);
}

/* Mode 6 / 6Index2 CompressSubset (src/Bc7CoreMode6.cpp:1334-1364): each
   later p-bit variant starts from the water left by the earlier ones. */
template<int kD, int MODE>
__device__ NEBC7_PASS int CompressSubsetSingle(SearchState& ss, const Area& ar, const AreaInfo& ai, const Params& P, const LevelTables& T,
	Ep& mc, int water, int lane)
{
	const int est[4] = { 0, 0, 0, 0 };
	const int pb[4] = { 0x0101, 0, 1, 1 << 8 };
	for (int v = 0; v < (ai.opaque ? 1 : 4); v++)
	{
		ChanList cl[4];
		if (InitLevels4<kD, MODE>(ss, 0, pb[v], ar, ai, P, T, water, est, cl, lane))
			water = TryV4<kD, MODE>(ss, 0, ar, ai, P, T, cl, mc, water, lane);
	}
	return water;
}

/* Mode 7 Subsets (src/Bc7CoreMode7.cpp:441-494). */
template<int kD>
__device__ NEBC7_PASS int SearchSubset7(SearchState& ss, const Area& ar, const AreaInfo& ai, const Params& P, const LevelTables& T,
	int water, const int est[4], Ep& best, bool& any, int lane)
{
	const int pb[4] = { 0x0101, 0, 1, 1 << 8 };
	ChanList cl[4][4];
	bool valid[4] = { false, false, false, false };
	for (int v = 0; v < (ai.opaque ? 1 : 4); v++)
		valid[v] = InitLevels4<kD, 7>(ss, v, pb[v], ar, ai, P, T, water, est, cl[v], lane);
	any = valid[0] || valid[1] || valid[2] || valid[3];
	for (int v = 0; v < 4; v++)
		if (valid[v])
			water = TryV4<kD, 7>(ss, v, ar, ai, P, T, cl[v], best, water, lane);
	return water;
}

template<int kD, int MODE>
__device__ NEBC7_PASS void RefineMode6(WarpState& st, SearchState& ss, CellRegs& R, const Params& P, const LevelTables& T, int lane)
{
	/* src/Bc7CoreMode6.cpp:1366-1381 */
	Ep mc = R.best[0];
	const int error = CompressSubsetSingle<kD, MODE>(ss, st.area1, R.a1, P, T, mc, R.errTotal, lane);
	if (R.errTotal > error)
	{
		R.errTotal = error;
		R.best[0] = mc;
	}
}

template<int kD>
__device__ NEBC7_PASS void FullMode6(WarpState& st, SearchState& ss, CellRegs& R, const Params& P, const LevelTables& T, int lane)
{
	/* src/Bc7CoreMode6.cpp:1398-1422 */
	if (R.personalMode == 6)
		return;
	const int step = R.denoiseStep;
	/* EstimateBest (src/Bc7CoreMode6.cpp:1383-1396): 0 without OPTION_PCA */
	const int line = P.pca ? PcaBound<kD>(st.area1, R.a1, P, R.a1.opaque ? 3 : 4, lane) : 0;
	if (line < R.errTotal - step)
	{
		Ep mc = 0;
		const int error = CompressSubsetSingle<kD, 6>(ss, st.area1, R.a1, P, T, mc, R.errTotal - step, lane);
		if (R.errTotal > error + step)
		{
			R.errTotal = error;
			R.best[0] = mc;
			R.bestMode = 6;
		}
	}
}

template<int kD>
__device__ NEBC7_PASS void RefineMode7(WarpState& st, SearchState& ss, CellRegs& R, const Params& P, const LevelTables& T, int lane)
{
	/* src/Bc7CoreMode7.cpp:496-557 */
	const int p = R.bestParam;
	Ep mc[2] = { R.best[0], R.best[1] };
	const int est[4] = { 0, 0, 0, 0 };
	const int w[4] = { P.wA, P.wG, P.wR, P.wB };
	int error = 0;
	for (int s = 0; s < 2; s++)
	{
		const AreaInfo ai = BuildSubset<kD>(st, R, P, st.sub[0], 2, p, s, lane);
		int water = AreaError<kD, 2>(st.sub[0], ai.active, mc[s], w, 2 * MaxColorError<kD>());
		water += TransparentError2(T, P, ai.count, ai.active, int(mc[s] & 0xFFFF));
		if (water)
		{
			bool any;
			Ep b = mc[s];
			const int r = SearchSubset7<kD>(ss, st.sub[0], ai, P, T, water, est, b, any, lane);
			if (any)
			{
				error += r;
				mc[s] = b;
			}
			else
				error += water;
		}
	}
	if (R.errTotal > error)
	{
		R.errTotal = error;
		R.best[0] = mc[0];
		R.best[1] = mc[1];
	}
}

/* EstimateLevels of mode 7 (src/Bc7CoreMode7.cpp:574-627). */
template<int kD>
__device__ NEBC7_PASS int EstimateLevels7(SearchState& ss, const Area& ar, const AreaInfo& ai, const Params& P, const LevelTables& T, int water,
	int est[4], int lane)
{
	int error = 0;
	if (error < water)
	{
		if (!ai.active)
		{
			est[0] = est[1] = est[2] = est[3] = 0;
			return 0;
		}
		if (!ai.opaque)
		{
			const int l0 = EstimateChannelLevels<kD>(ar, ai, 0, P.wA, water - error, 6, false, kReducedByDiff ? T.d2v8 : T.d2v6, kReducedByDiff,
				T.c2v6, ss.uniq, lane);
			est[0] = l0;
			error += l0;
		}
		else
			est[0] = 0;
		const int wts[4] = { P.wA, P.wG, P.wR, P.wB };
		for (int c = 1; c < 4; c++)
		{
			if (!(error < water))
				return water;
			const int l = EstimateChannelLevels<kD>(ar, ai, c, wts[c], water - error, 6, true, kReducedByDiff ? T.d2v8 : T.d2v6, kReducedByDiff,
				T.c2v6, ss.uniq, lane);
			est[c] = l;
			error += l;
		}
		if (error < water)
			return error;
	}
	return water;
}

/* The partition search of mode 7 from its estimates (the second loop of
   src/Bc7CoreMode7.cpp:629-725): partition p with the principal-axis bounds
   line1, line2 (0 without OPTION_PCA).  Returns true when the search ends
   the full pass. */
template<int kD>
__device__ __forceinline__ bool Mode7Partition(WarpState& st, SearchState& ss, CellRegs& R, const Params& P, const LevelTables& T,
	int p, int line1, int line2, int lane)
{
	const int step = R.denoiseStep;
	Ep mc[2] = { 0, 0 };
	int e1[4], e2[4];
	const AreaInfo a1 = BuildSubset<kD>(st, R, P, st.sub[0], 2, p, 0, lane);
	const AreaInfo a2 = BuildSubset<kD>(st, R, P, st.sub[1], 2, p, 1, lane);
	int w1 = R.errTotal - step - line2;
	line1 = max(line1, EstimateLevels7<kD>(ss, st.sub[0], a1, P, T, w1, e1, lane));
	if (line1 < w1)
	{
		int w2 = w1 - line1;
		line2 = max(line2, EstimateLevels7<kD>(ss, st.sub[1], a2, P, T, w2, e2, lane));
		if (line2 < w2)
		{
			w1 = R.errTotal - step - line2;
			bool any;
			int error = SearchSubset7<kD>(ss, st.sub[0], a1, P, T, w1, e1, mc[0], any, lane);
			if (any && error < w1)
			{
				w2 = R.errTotal - step - error;
				const int r2 = SearchSubset7<kD>(ss, st.sub[1], a2, P, T, w2, e2, mc[1], any, lane);
				if (any)
				{
					error += r2;
					if (R.errTotal > error + step)
					{
						R.errTotal = error;
						R.best[0] = mc[0];
						R.best[1] = mc[1];
						R.bestParam = p;
						R.bestMode = 7;
						if (error <= 0)
							return true;
					}
				}
			}
		}
	}
	return false;
}

/* EstimateBest of mode 7 (src/Bc7CoreMode7.cpp:559-572): the principal-axis
   bound over G, R, B for an opaque area, over A, G, R, B otherwise. */
template<int kD>
__device__ __forceinline__ int EstimateBest(const Area& ar, const AreaInfo& ai, const Params& P, int lane)
{
	return PcaBound<kD>(ar, ai, P, ai.opaque ? 3 : 4, lane);
}

template<int kD>
__device__ NEBC7_PASS void FullMode7(WarpState& st, SearchState& ss, CellRegs& R, const Params& P, const LevelTables& T, int lane,
	int from = 0)
{
	/* src/Bc7CoreMode7.cpp:629-725; without OPTION_PCA every partition enters
	   with estimate step (ties keep index order), and the search may resume
	   at partition `from` */
	const int step = R.denoiseStep;
	if (!P.pca)
	{
		for (int p = from; p < 64; p++)
		{
			if (R.personalMode == 7 && R.personalParam == p)
				continue;
			if (!(0 < R.errTotal - step))
				continue;
			if (!(step < R.errTotal))
				continue;
			if (Mode7Partition<kD>(st, ss, R, P, T, p, 0, 0, lane))
				return;
		}
		return;
	}
	int count = 0;
	for (int p = 0; p < 64; p++)
	{
		if (R.personalMode == 7 && R.personalParam == p)
			continue;
		const AreaInfo a1 = BuildSubset<kD>(st, R, P, st.sub[0], 2, p, 0, lane);
		const int water1 = R.errTotal - step;
		const int line1 = EstimateBest<kD>(st.sub[0], a1, P, lane);
		if (line1 < water1)
		{
			const AreaInfo a2 = BuildSubset<kD>(st, R, P, st.sub[1], 2, p, 1, lane);
			const int line2 = EstimateBest<kD>(st.sub[1], a2, P, lane);
			if (line2 < water1 - line1)
			{
				if (lane == 0)
				{
					ss.lines[p][0] = line1;
					ss.lines[p][1] = line2;
					ss.order[count] = make_int2(line1 + line2 + step, p);
				}
				count++;
			}
		}
		__syncwarp();
	}
	__syncwarp();
	StableSortOrder(ss.order, count, lane);
	for (int i = 0; i < count; i++)
	{
		const int2 o = ss.order[i];
		if (o.x < R.errTotal && Mode7Partition<kD>(st, ss, R, P, T, o.y, ss.lines[o.y][0], ss.lines[o.y][1], lane))
			return;
	}
}

/* ---------------------------------------------------------------------- */
/* Modes 4 and 5: rotation, separate color / alpha-slot indices            */
/* ---------------------------------------------------------------------- */

template<int kD, int MODE, int CB, int AB>
__device__ NEBC7_SHARED int TryVariantsRot(const Area& ar, const AreaInfo& ai, const Params& P, const int2* const* Ls, const ChanList* cl,
	Ep& bestStorage, int water, int rot, int lane)
{
	const int minA = cl[0].minErr, minG = cl[1].minErr, minR = cl[2].minErr, minB = cl[3].minErr;
	if (minA + minG + minR + minB >= water)
		return water;
	const int nA = (rot == 0) ? 1 : cl[0].count;
	const int nG = (rot == 2) ? 1 : cl[1].count;
	const int nR = (rot == 1) ? 1 : cl[2].count;
	const int nB = (rot == 3) ? 1 : cl[3].count;
	const int wAG[4] = { P.wA, P.wG, 0, 0 };
	const int wAR[4] = { P.wA, 0, P.wR, 0 };
	const int wAGR[4] = { P.wA, P.wG, P.wR, 0 };
	const int wAGB[4] = { P.wA, P.wG, 0, P.wB };
	const int wAGRB[4] = { P.wA, P.wG, P.wR, P.wB };
	const int2* LA = Ls[0];
	const int2* LG = Ls[1];
	const int2* LR = Ls[2];
	const int2* LB = Ls[3];
	const int colB = lane < nB ? LB[lane].y : 0;
	const int eBbase = lane < nB ? LB[lane].x : kBig;
	for (int iA = 0; iA < nA; iA++)
	{
		const int eA = LA[iA].x;
		if (eA + minG + minR + minB >= water)
			break;
		const int cA = LA[iA].y;
		int memAR = kBig, pairAG = kBig;
		if ((rot == 2 || rot == 3) && lane < nR)
			memAR = RotErrorW<kD, CB, AB, MODE == 4>(ar, ai, Ep2(0, cA, 2, LR[lane].y), rot, wAR, water - minG - minB);
		if ((rot == 1 || rot == 3) && lane < nG)
			pairAG = RotErrorW<kD, CB, AB, MODE == 4>(ar, ai, Ep2(0, cA, 1, LG[lane].y), rot, wAG, water - minR - minB);
		for (int iG = 0; iG < nG; iG++)
		{
			int eG = LG[iG].x + eA;
			if (eG + minR + minB >= water)
				break;
			const int cG = LG[iG].y;
			if (rot == 1 || rot == 3)
			{
				eG = __shfl_sync(kFull, pairAG, iG);
				if (eG + minR + minB >= water)
					continue;
			}
			const Ep baseAG = Ep2(0, cA, 1, cG);
			int memAGB = kBig, pairAGR = kBig;
			if (rot != 3 && lane < nB)
				memAGB = RotErrorW<kD, CB, AB, MODE == 4>(ar, ai, EpSetCh(baseAG, 3, LB[lane].y), rot, wAGB, water - minR);
			if ((rot == 0 || rot == 3) && lane < nR)
				pairAGR = RotErrorW<kD, CB, AB, MODE == 4>(ar, ai, EpSetCh(baseAG, 2, LR[lane].y), rot, wAGR, water - minB);
			for (int iR = 0; iR < nR; iR++)
			{
				int eR = LR[iR].x + eG;
				if (eR + minB >= water)
					break;
				const int cR = LR[iR].y;
				if (rot == 2 || rot == 3)
				{
					const int ear = __shfl_sync(kFull, memAR, iR);
					if (ear + minG + minB >= water)
						continue;
					if (rot == 2)
						eR = ear + LG[iG].x;
				}
				if (rot == 0 || rot == 3)
				{
					eR = __shfl_sync(kFull, pairAGR, iR);
					if (eR + minB >= water)
						continue;
				}
				const Ep baseAGR = EpSetCh(baseAG, 2, cR);
				const bool valid = lane < nB;
				const int brk = valid ? eBbase + eR : kBig;
				const int skip = (valid && rot != 3) ? memAGB + minR : brk;
				int err = kBig;
				if (valid && brk < water && skip < water)
				{
					if (rot == 1)
						err = memAGB + LR[iR].x;
					else if (rot == 3)
						err = brk;
					else
						err = RotErrorW<kD, CB, AB, MODE == 4>(ar, ai, EpSetCh(baseAGR, 3, colB), rot, wAGRB, water);
				}
				const int jl = ReplayInner(valid, brk, skip, err, water, lane);
				if (jl >= 0)
					bestStorage = EpSwapRot(EpSetCh(baseAGR, 3, __shfl_sync(kFull, colB, jl)), rot);
			}
		}
	}
	return water;
}

/* Subset InitLevels of modes 4 / 5 (src/Bc7CoreMode4.cpp:1264-1322, :1505-1563,
   src/Bc7CoreMode5.cpp:628-686) + TryVariants. */
template<int kD, int MODE>
__device__ NEBC7_PASS int CompressRotSubset(WarpState& st, SearchState& ss, const CellRegs& R, const Params& P, const LevelTables& T,
	Ep& mcStorage, int water, int rotation, int lane)
{
	const Area& ar = st.area1;
	const AreaInfo& ai = R.a1;
	const bool idx32 = MODE == 4 && (rotation & 4);
	const int a = RotChannel(rotation);
	int cbits, abits;
	const uint8_t *ctab, *atab;
	if (MODE == 4)
	{
		cbits = 5;
		abits = 6;
		ctab = kReducedByDiff ? (idx32 ? T.d3v8 : T.d2v8) : (idx32 ? T.d3v5 : T.d2v5);
		atab = kReducedByDiff ? (idx32 ? T.d2v8 : T.d3v8) : (idx32 ? T.d2v6 : T.d3v6);
	}
	else
	{
		cbits = 7;
		abits = 8;
		ctab = kReducedByDiff ? T.d2v8 : T.d2v7;
		atab = T.d2v8;
	}
	const int wts[4] = { P.wA, P.wG, P.wR, P.wB };
	ChanList cl[4];
	int used = 0;
	for (int c = 0; c < 4; c++)
	{
		if (c == 0 && ai.opaque)
			cl[0] = ZeroList(ss.lists[0][0], 0xFFFF, lane);
		else if (c == a)
			cl[c] = ChannelLevelsSingle<kD>(ss.lists[0][c], ar, ai, c, wts[c], water - used, abits, c != 0, atab, kReducedByDiff || abits == 8,
				ss.uniq, lane);
		else
			cl[c] = ChannelLevels<kD, false>(ss.lists[0][c], ar, ai, c, wts[c], water - used, cbits, -1, c != 0, ctab, kReducedByDiff, 32,
				ss.uniq, lane);
		used += cl[c].minErr;
		if (used >= water)
			return water;
	}
	const int2* Ls[4] = { ss.lists[0][0], ss.lists[0][1], ss.lists[0][2], ss.lists[0][3] };
	const int rot = rotation & 3;
	if (MODE == 5)
		return TryVariantsRot<kD, 5, 2, 2>(ar, ai, P, Ls, cl, mcStorage, water, rot, lane);
	if (idx32)
		return TryVariantsRot<kD, 4, 3, 2>(ar, ai, P, Ls, cl, mcStorage, water, rot, lane);
	return TryVariantsRot<kD, 4, 2, 3>(ar, ai, P, Ls, cl, mcStorage, water, rot, lane);
}

template<int kD>
__device__ NEBC7_PASS void RefineMode4(WarpState& st, SearchState& ss, CellRegs& R, const Params& P, const LevelTables& T, int lane)
{
	/* src/Bc7CoreMode4.cpp:1795-1822 */
	int rotation = R.bestParam;
	for (int i = 0; i < 2; i++, rotation ^= 4)
	{
		Ep mc = 0;
		const int error = CompressRotSubset<kD, 4>(st, ss, R, P, T, mc, R.errTotal, rotation, lane);
		if (R.errTotal > error)
		{
			R.errTotal = error;
			R.best[0] = mc;
			R.bestParam = rotation;
			if (error <= 0)
				break;
		}
	}
}

template<int kD>
__device__ NEBC7_PASS void RefineMode5(WarpState& st, SearchState& ss, CellRegs& R, const Params& P, const LevelTables& T, int lane)
{
	/* src/Bc7CoreMode5.cpp:890-911 */
	Ep mc = 0;
	const int error = CompressRotSubset<kD, 5>(st, ss, R, P, T, mc, R.errTotal, R.bestParam, lane);
	if (R.errTotal > error)
	{
		R.errTotal = error;
		R.best[0] = mc;
	}
}

template<int kD, int MODE>
__device__ NEBC7_PASS void FullRot(WarpState& st, SearchState& ss, CellRegs& R, const Params& P, const LevelTables& T, int lane,
	int from = 0)
{
	/* src/Bc7CoreMode4.cpp:1824-1857, src/Bc7CoreMode5.cpp:913-946; the
	   search may resume at choice `from` */
	const int step = R.denoiseStep;
	constexpr int NR = MODE == 4 ? 8 : 4;
	for (int ri = from; ri < NR; ri++)
	{
		const int rotation = MODE == 4 ? c_rot4[ri] : c_rot5[ri];
		if (MODE == 4 && R.personalMode == 4 && !((R.personalParam ^ rotation) & 3))
			continue;
		if (MODE == 5 && R.personalMode == 5 && R.personalParam == rotation)
			continue;
		Ep mc = 0;
		int error = step;
		if (error < R.errTotal)
			error += CompressRotSubset<kD, MODE>(st, ss, R, P, T, mc, R.errTotal - error, rotation, lane);
		if (R.errTotal > error)
		{
			R.errTotal = error - step;
			R.best[0] = mc;
			R.bestParam = rotation;
			R.bestMode = MODE;
			if (error <= step)
				break;
		}
	}
}

/* ---------------------------------------------------------------------- */
/* The normal / slow pass chain (src/Bc7Core.cpp:1604-1745)                */
/* ---------------------------------------------------------------------- */

template<int kD>
__device__ void NormalPasses(WarpState& st, SearchState& ss, CellRegs& R, const Params& P, const LevelTables& T, int lane)
{
	const int OA = R.opaqueAlphaError;
	const int step = R.denoiseStep;

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

	if (R.a1.opaque)
	{
		if (R.errTotal > OA + step)
		{
			FullThreeSubsets<kD, 2>(st, ss, R, P, T, lane);
			if (R.errTotal > OA + step)
			{
				FullThreeSubsets<kD, 0>(st, ss, R, P, T, lane);
				if (P.doSlow && R.errTotal > OA + step)
				{
					FullTwoSubsets<kD, 1>(st, ss, R, P, T, lane);
					if (R.errTotal > OA + step)
					{
						FullTwoSubsets<kD, 3>(st, ss, R, P, T, lane);
						if (R.errTotal > step)
						{
							FullRot<kD, 5>(st, ss, R, P, T, lane);
							if (R.errTotal > step)
							{
								FullRot<kD, 4>(st, ss, R, P, T, lane);
								if (R.errTotal > step)
								{
									FullMode7<kD>(st, ss, R, P, T, lane);
									if (R.errTotal > step)
										FullMode6<kD>(st, ss, R, P, T, lane);
								}
							}
						}
					}
				}
			}
		}
	}
	else
	{
		if (R.errTotal > step)
		{
			FullRot<kD, 5>(st, ss, R, P, T, lane);
			if (R.errTotal > step)
			{
				FullRot<kD, 4>(st, ss, R, P, T, lane);
				if (R.errTotal > step)
				{
					FullMode7<kD>(st, ss, R, P, T, lane);
					if (P.doSlow && R.errTotal > step)
						FullMode6<kD>(st, ss, R, P, T, lane);
				}
			}
		}
	}
}

} // namespace nebc7
