/*
 * BC7 block encoder for sm_103a -- bounding-box ("fast") mode passes and the
 * final index selection / BPTC packing of every mode.
 *
 * A fast pass (reference ModeN::CompressBlockFast) tries every partition or
 * rotation of a mode with endpoints quantised from the subset's oriented
 * bounds, in a fixed order, taking a candidate only when it beats the
 * running error (which then drops by the denoise step).  Here each lane
 * evaluates whole candidates (lane = partition or rotation) with exact
 * errors, the errors go to shared memory, and one warp-uniform scan replays
 * the reference's acceptance order: a candidate with error E is taken iff
 * E < T, after which T = E - step, with the same early stop.  The
 * reference's early-exit partial sums only ever decide rejections, which
 * the exact errors decide the same way.
 */
#pragma once

#include "bc7_block.cuh"

namespace nebc7 {

/* ---------------------------------------------------------------------- */
/* Endpoint quantisation from bounds                                      */
/* ---------------------------------------------------------------------- */

__device__ __forceinline__ Ep EpFromLanes(const uint16_t b[8])
{
	Ep e = 0;
	for (int i = 0; i < 8; i++)
		e |= uint64_t(b[i] & 0xFF) << (8 * i);
	return e;
}

/* mode 0: 4 bits + unique p-bit taken from G's bit 3 (src/Bc7CoreMode0.cpp:169-187) */
__device__ __forceinline__ Ep QuantMode0(const uint16_t b[8])
{
	const int p0 = b[2] & 8, p1 = b[3] & 8;
	Ep e = 0;
	for (int i = 0; i < 8; i++)
	{
		int v = b[i] & 0xF0;
		v |= v >> 5;
		v |= (i & 1) ? p1 : p0;
		e |= uint64_t(v & 0xFF) << (8 * i);
	}
	return e;
}

/* mode 1: 6 bits + shared p-bit, p = 0 (src/Bc7CoreMode1.cpp:141-174) */
__device__ __forceinline__ Ep QuantMode1(const uint16_t b[8])
{
	Ep e = 0;
	for (int i = 0; i < 8; i++)
	{
		int v = b[i] & 0xFC;
		v |= v >> 7;
		e |= uint64_t(v & 0xFF) << (8 * i);
	}
	return e;
}

/* mode 2: 5 bits (src/Bc7CoreMode2.cpp:150-163) */
__device__ __forceinline__ Ep QuantMode2(const uint16_t b[8])
{
	Ep e = 0;
	for (int i = 0; i < 8; i++)
	{
		int v = b[i] & 0xF8;
		v |= v >> 5;
		e |= uint64_t(v & 0xFF) << (8 * i);
	}
	return e;
}

/* mode 3: 7 bits + unique p-bit from G's bit 0 (src/Bc7CoreMode3.cpp:140-156) */
__device__ __forceinline__ Ep QuantMode3(const uint16_t b[8])
{
	const int p0 = b[2] & 1, p1 = b[3] & 1;
	Ep e = 0;
	for (int i = 0; i < 8; i++)
		e |= uint64_t(((b[i] & 0xFE) | ((i & 1) ? p1 : p0)) & 0xFF) << (8 * i);
	return e;
}

/* mode 7: 5 bits + unique p-bit from A's bit 2 (src/Bc7CoreMode7.cpp:161-184) */
__device__ __forceinline__ Ep QuantMode7(const uint16_t b[8])
{
	const int p0 = b[0] & 4, p1 = b[1] & 4;
	Ep e = 0;
	for (int i = 0; i < 8; i++)
	{
		int v = b[i] & 0xF8;
		v |= v >> 6;
		v |= (i & 1) ? p1 : p0;
		e |= uint64_t(v & 0xFF) << (8 * i);
	}
	return e;
}

/* modes 6 / 6Index2: 7 bits + unique p-bit from A's bit 0
   (src/Bc7CoreMode6.cpp:1077-1098) */
__device__ __forceinline__ Ep QuantMode6(const uint16_t b[8])
{
	const int p0 = b[0] & 1, p1 = b[1] & 1;
	Ep e = 0;
	for (int i = 0; i < 8; i++)
		e |= uint64_t(((b[i] & 0xFE) | ((i & 1) ? p1 : p0)) & 0xFF) << (8 * i);
	return e;
}

/* mode 4 in block (storage) order: alpha slot 6 bits, colors 5 bits
   (src/Bc7CoreMode4.cpp:1195-1223) */
__device__ __forceinline__ Ep QuantMode4(const uint16_t b[8], int rotation)
{
	const Ep img = EpFromLanes(b);
	const Ep s = EpSwapRot(img, rotation);
	Ep e = 0;
	for (int i = 0; i < 8; i++)
	{
		const int x = EpGet(s, i);
		const int v = i < 2 ? ((x & 0xFC) | (x >> 6)) : ((x & 0xF8) | (x >> 5));
		e |= uint64_t(v & 0xFF) << (8 * i);
	}
	return e;
}

/* mode 5 in block order: alpha slot 8 bits, colors 7 bits
   (src/Bc7CoreMode5.cpp:569-587) */
__device__ __forceinline__ Ep QuantMode5(const uint16_t b[8], int rotation)
{
	const Ep img = EpFromLanes(b);
	const Ep s = EpSwapRot(img, rotation);
	Ep e = 0;
	for (int i = 0; i < 8; i++)
	{
		const int x = EpGet(s, i);
		const int v = i < 2 ? x : ((x & 0xFE) | (x >> 7));
		e |= uint64_t(v & 0xFF) << (8 * i);
	}
	return e;
}

/* ---------------------------------------------------------------------- */
/* Subset membership                                                      */
/* ---------------------------------------------------------------------- */

__device__ __forceinline__ uint32_t Member(uint32_t part, int s)
{
	uint32_t m = 0;
#pragma unroll
	for (int i = 0; i < 16; i++)
		m |= uint32_t(((part >> (2 * i)) & 3) == uint32_t(s)) << i;
	return m;
}

__device__ __forceinline__ int Anchor(int ns, int p, int s)
{
	if (s == 0)
		return 0;
	if (ns == 2)
		return c_anchor22[p];
	return s == 1 ? c_anchor23[p] : c_anchor33[p];
}

/* ---------------------------------------------------------------------- */
/* Fast passes                                                            */
/* ---------------------------------------------------------------------- */

/* Replays the reference's acceptance order over errors in st.scan[0..n):
   returns the index of the last accepted candidate (or -1) and updates T. */
__device__ __forceinline__ int AcceptScan(const WarpState& st, int n, int& T, int step, int stopAt)
{
	int won = -1;
	for (int i = 0; i < n; i++)
	{
		const int E = st.scan[i];
		if (E < T)
		{
			T = E - step;
			won = i;
			if (E <= stopAt)
				break;
		}
	}
	return won;
}

/* Modes 0-3: opaque subsets, errors over G, R, B. */
template<int kD, int MODE>
__device__ NEBC7_ONCE void FastOpaque(WarpState& st, CellRegs& R, const Params& P, int lane)
{
	constexpr int NS = (MODE == 0 || MODE == 2) ? 3 : 2;
	constexpr int NP = MODE == 0 ? 16 : 64;
	constexpr int IB = (MODE == 0 || MODE == 1) ? 3 : 2;
	const int step = R.denoiseStep;
	const int wGRB[4] = { 0, P.wG, P.wR, P.wB };

	Ep keep[2][3];
	for (int round = 0; round < (NP + 31) / 32; round++)
	{
		const int p = round * 32 + lane;
		int E = 0x7FFFFFFF;
		Ep ep[3] = { 0, 0, 0 };
		if (p < NP)
		{
			const uint32_t part = NS == 3 ? c_part3[p] : c_part2[p];
			E = R.opaqueAlphaError + step;
			for (int s = 0; s < NS; s++)
			{
				const uint32_t member = Member(part, s);
				const AreaInfo ai = AreaStats(st, R, P, member);
				const uint32_t act = member & R.visible;
				int e;
				if (MODE == 0)
				{
					ep[s] = QuantMode0(ai.bounds);
					e = SubsetErrorMask<kD, 3>(st, act, ep[s], wGRB);
				}
				else if (MODE == 1)
				{
					ep[s] = QuantMode1(ai.bounds);
					const int e0 = SubsetErrorMask<kD, 3>(st, act, ep[s], wGRB);
					const Ep ep1 = ep[s] | 0x0202020202020202ull;
					const int e1 = SubsetErrorMask<kD, 3>(st, act, ep1, wGRB);
					e = e0;
					if (e1 < e0)
					{
						e = e1;
						ep[s] = ep1;
					}
				}
				else if (MODE == 2)
				{
					ep[s] = QuantMode2(ai.bounds);
					e = SubsetErrorMask<kD, 2>(st, act, ep[s], wGRB);
				}
				else
				{
					ep[s] = QuantMode3(ai.bounds);
					e = SubsetErrorMask<kD, 2>(st, act, ep[s], wGRB);
				}
				E += e;
			}
		}
		st.scan[p & 63] = E;
		for (int s = 0; s < 3; s++)
			keep[round & 1][s] = ep[s];
	}
	__syncwarp();
	int T = R.errTotal;
	const int won = AcceptScan(st, NP, T, step, R.opaqueAlphaError + step);
	__syncwarp();
	if (won >= 0)
	{
		const int owner = won & 31;
		const int round = won >> 5;
		R.errTotal = T;
		for (int s = 0; s < NS; s++)
		{
			const Ep v = round ? keep[1][s] : keep[0][s];
			R.best[s] = __shfl_sync(kFull, v, owner);
		}
		R.bestParam = won;
		R.bestMode = MODE;
	}
}

/* Mode 7: two RGBA subsets with the transparent-alpha term. */
template<int kD>
__device__ NEBC7_ONCE void FastMode7(WarpState& st, CellRegs& R, const Params& P, const LevelTables& T, int lane)
{
	const int step = R.denoiseStep;
	const int w[4] = { P.wA, P.wG, P.wR, P.wB };
	Ep keep[2][2];
	for (int round = 0; round < 2; round++)
	{
		const int p = round * 32 + lane;
		int E = step;
		Ep ep[2];
		for (int s = 0; s < 2; s++)
		{
			const uint32_t member = Member(c_part2[p], s);
			const AreaInfo ai = AreaStats(st, R, P, member);
			ep[s] = QuantMode7(ai.bounds);
			const int ea = TransparentError2(T, P, ai.count, ai.active, int(ep[s] & 0xFFFF));
			E += ea + SubsetErrorMask<kD, 2>(st, member & R.visible, ep[s], w);
		}
		st.scan[p] = E;
		keep[round][0] = ep[0];
		keep[round][1] = ep[1];
	}
	__syncwarp();
	int Tt = R.errTotal;
	const int won = AcceptScan(st, 64, Tt, step, step);
	__syncwarp();
	if (won >= 0)
	{
		const int owner = won & 31;
		const int round = won >> 5;
		R.errTotal = Tt;
		for (int s = 0; s < 2; s++)
			R.best[s] = __shfl_sync(kFull, round ? keep[1][s] : keep[0][s], owner);
		R.bestParam = won;
		R.bestMode = 7;
	}
}

/* Modes 4 and 5: one subset (Area1) per rotation. */
template<int kD, int MODE>
__device__ NEBC7_ONCE void FastRot(WarpState& st, CellRegs& R, const Params& P, int lane)
{
	constexpr int NR = MODE == 4 ? 8 : 4;
	const int step = R.denoiseStep;
	const int w[4] = { P.wA, P.wG, P.wR, P.wB };
	Ep mine = 0;
	if (lane < NR)
	{
		const int rotation = MODE == 4 ? c_rot4[lane] : c_rot5[lane];
		int e;
		if (MODE == 4)
		{
			mine = QuantMode4(R.a1.bounds, rotation);
			const Ep img = EpSwapRot(mine, rotation);
			if (rotation & 4)
				e = RotErrorExact<kD, 3, 2, true>(st, R, img, rotation, w);
			else
				e = RotErrorExact<kD, 2, 3, true>(st, R, img, rotation, w);
		}
		else
		{
			mine = QuantMode5(R.a1.bounds, rotation);
			const Ep img = EpSwapRot(mine, rotation);
			e = RotErrorExact<kD, 2, 2, false>(st, R, img, rotation, w);
		}
		st.scan[lane] = step + e;
	}
	__syncwarp();
	int T = R.errTotal;
	const int won = AcceptScan(st, NR, T, step, step);
	__syncwarp();
	if (won >= 0)
	{
		R.errTotal = T;
		R.best[0] = __shfl_sync(kFull, mine, won);
		R.bestParam = MODE == 4 ? c_rot4[won] : c_rot5[won];
		R.bestMode = MODE;
	}
}

/* Modes 6 and 6Index2: one candidate. */
template<int kD, bool INDEX2>
__device__ NEBC7_ONCE void FastMode6(WarpState& st, CellRegs& R, const Params& P, const LevelTables& T)
{
	const int step = R.denoiseStep;
	const int w[4] = { P.wA, P.wG, P.wR, P.wB };
	const Ep ep = QuantMode6(R.a1.bounds);
	int E = step;
	if (INDEX2)
		E += TransparentError2(T, P, 16, R.a1.active, int(ep & 0xFFFF)) + SubsetErrorMask<kD, 2>(st, R.visible, ep, w);
	else
		E += TransparentError4(T, P, 16, R.a1.active, int(ep & 0xFFFF)) + SubsetErrorMask<kD, 4>(st, R.visible, ep, w);
	if (E < R.errTotal)
	{
		R.errTotal = E - step;
		R.best[0] = ep;
		R.bestMode = INDEX2 ? 9 : 6;
	}
}

/* ---------------------------------------------------------------------- */
/* Final index selection and packing                                      */
/* ---------------------------------------------------------------------- */

struct BitOut
{
	uint64_t lo = 0, hi = 0;
	int pos = 0;

	__device__ void Put(uint64_t v, int n)
	{
		v &= (uint64_t(1) << n) - 1;
		if (pos >= 64)
			hi |= v << (pos - 64);
		else
		{
			lo |= v << pos;
			if (pos + n > 64)
				hi |= v >> (64 - pos);
		}
		pos += n;
	}

	/* per-pixel indices of `bits` each (pixel 0 first); anchors drop their
	   zero MSB */
	__device__ void PutIndices(uint64_t indices, int bits, int a0, int a1, int a2)
	{
		for (int i = 0; i < 16; i++)
		{
			const bool anchor = (i == a0 || i == a1 || i == a2);
			Put((indices >> (i * bits)) & ((uint64_t(1) << bits) - 1), anchor ? bits - 1 : bits);
		}
	}
};

template<int BITS>
__device__ __forceinline__ void Levels4(Ep ep, int vals[1 << BITS][4])
{
	const int* w = InterpWeights(BITS);
#pragma unroll
	for (int k = 0; k < (1 << BITS); k++)
#pragma unroll
		for (int c = 0; c < 4; c++)
			vals[k][c] = Interp(EpGet(ep, 2 * c), EpGet(ep, 2 * c + 1), w[k]);
}

/* Index selection of one subset: indices land at their pixel positions.
   Optionally also returns the unweighted alpha error of the chosen levels
   (the <opaque=false> variants, src/SnippetComputeOpaqueSubset2.h:660-684). */
template<int kD, int BITS>
__device__ int SubsetTable(WarpState& st, const Area& ar, const AreaInfo& ai, const Params& P, const int w[4], const int vals[1 << BITS][4],
	uint64_t& indices, int* alphaErr, int lane)
{
	const int err = ComputeSubsetTable<kD, (1 << BITS)>(st, ar, ai, P, w, vals, lane);
	uint64_t mine = 0;
	int ea = 0;
	if (lane < ai.count)
	{
		mine = uint64_t(unsigned(st.best[lane])) << (ar.idx[lane] * BITS);
		int da = vals[st.best[lane]][0] - int(ar.px[lane][0]);
		da = da < 0 ? -da : da;
		da = kD ? (da >> kD) : (da > 127 ? 127 : da);
		ea = da * da;
	}
	/* OR-reduce the per-pixel index fields */
	for (int o = 16; o > 0; o >>= 1)
		mine |= __shfl_xor_sync(kFull, mine, o);
	indices |= mine;
	if (alphaErr)
		*alphaErr = int(__reduce_add_sync(kFull, unsigned(ea)));
	__syncwarp();
	return err;
}

/* AreaReduceTable2/3 (src/Bc7Core.cpp:511-549): if the anchor's index MSB is
   set, invert the subset's indices and swap its endpoints. */
__device__ __forceinline__ void ReduceTable(uint32_t member, int anchor, int bits, Ep& ep, uint64_t& indices)
{
	if (indices & (uint64_t(1) << (anchor * bits + bits - 1)))
	{
		uint64_t mask = 0;
		for (int i = 0; i < 16; i++)
			if ((member >> i) & 1)
				mask |= ((uint64_t(1) << bits) - 1) << (i * bits);
		indices ^= mask;
		ep = EpSwapEnds(ep);
	}
}

/* Final packing of modes 0-3 and 7 (src/Bc7CoreMode{0,1,2,3,7}.cpp
   FinalPackBlock + ComposeBlock). */
template<int kD, int MODE>
__device__ void FinalPackPartitioned(WarpState& st, CellRegs& R, const Params& P, uint64_t& lo, uint64_t& hi, int lane)
{
	constexpr int NS = (MODE == 0 || MODE == 2) ? 3 : 2;
	constexpr int IB = (MODE == 0 || MODE == 1) ? 3 : 2;
	const int p = R.bestParam;
	const uint32_t part = NS == 3 ? c_part3[p] : c_part2[p];
	const int w[4] = { P.wA, P.wG, P.wR, P.wB };

	uint64_t indices = 0;
	int total = 0, alpha = 0;
	Ep ep[3];
	for (int s = 0; s < NS; s++)
	{
		const uint32_t member = Member(part, s);
		const int anchor = Anchor(NS, p, s);
		AreaInfo ai = AreaStats(st, R, P, member);
		ai.zero = anchor;
		BuildAreaList(st.sub[0], st, R, member, anchor, lane);
		ep[s] = R.best[s];
		if (MODE != 7)
			ep[s] |= 0xFFFF;
		int vals[1 << IB][4];
		Levels4<IB>(ep[s], vals);
		int ea = 0;
		total += SubsetTable<kD, IB>(st, st.sub[0], ai, P, w, vals, indices, MODE == 7 ? &ea : nullptr, lane);
		alpha += ea * P.wA;
	}
	if (MODE == 7)
	{
		R.errAlpha = alpha;
		R.errTotal = total;
	}
	else
	{
		R.errAlpha = R.opaqueAlphaError;
		R.errTotal = total;
	}
	for (int s = 0; s < NS; s++)
		ReduceTable(Member(part, s), Anchor(NS, p, s), IB, ep[s], indices);

	BitOut bw;
	bw.Put(uint64_t(1) << MODE, MODE + 1);
	bw.Put(uint64_t(p), MODE == 0 ? 4 : 6);
	const int cbits = MODE == 0 ? 4 : (MODE == 1 ? 6 : (MODE == 2 ? 5 : (MODE == 3 ? 7 : 5)));
	const int cshift = 8 - cbits;
	const int order[4] = { 2, 1, 3, 0 };
	for (int oc = 0; oc < (MODE == 7 ? 4 : 3); oc++)
		for (int s = 0; s < NS; s++)
			for (int k = 0; k < 2; k++)
				bw.Put(uint64_t(EpGet(ep[s], 2 * order[oc] + k) >> cshift), cbits);
	if (MODE == 0)
	{
		for (int s = 0; s < 3; s++)
			for (int k = 0; k < 2; k++)
				bw.Put(uint64_t((EpGet(ep[s], 2 + k) >> 3) & 1), 1);
	}
	else if (MODE == 1)
	{
		for (int s = 0; s < 2; s++)
			bw.Put(uint64_t((EpGet(ep[s], 2) >> 1) & 1), 1);
	}
	else if (MODE == 3)
	{
		for (int s = 0; s < 2; s++)
			for (int k = 0; k < 2; k++)
				bw.Put(uint64_t(EpGet(ep[s], 2 + k) & 1), 1);
	}
	else if (MODE == 7)
	{
		for (int s = 0; s < 2; s++)
			for (int k = 0; k < 2; k++)
				bw.Put(uint64_t((EpGet(ep[s], k) >> 2) & 1), 1);
	}
	bw.PutIndices(indices, IB, 0, Anchor(NS, p, 1), NS == 3 ? Anchor(NS, p, 2) : -1);
	lo = bw.lo;
	hi = bw.hi;
}

/* Final packing of modes 4 and 5 (src/Bc7CoreMode4.cpp:841-1193,
   src/Bc7CoreMode5.cpp:403-567). */
template<int kD, int MODE>
__device__ void FinalPackRot(WarpState& st, CellRegs& R, const Params& P, uint64_t& lo, uint64_t& hi, int lane)
{
	const int rotation = R.bestParam;
	const bool idx32 = MODE == 4 && (rotation & 4);
	const int a = RotChannel(rotation);
	const Ep epS = R.best[0];
	const Ep epI = EpSwapRot(epS, rotation);
	AreaInfo ai = R.a1;
	ai.zero = 0;

	int wc[4] = { P.wA, P.wG, P.wR, P.wB };
	int wa[4] = { 0, 0, 0, 0 };
	wa[a] = wc[a];
	wc[a] = 0;

	uint64_t idxC = 0, idxA = 0;
	int errC, errA, eaC = 0, eaA = 0;
	if (MODE == 4 && !idx32)
	{
		int vc[4][4], va[8][4];
		Levels4<2>(epI, vc);
		Levels4<3>(epI, va);
		for (int k = 0; k < 4; k++)
			vc[k][a] = 0;
		for (int k = 0; k < 8; k++)
			for (int c = 0; c < 4; c++)
				if (c != a)
					va[k][c] = 0;
		errC = SubsetTable<kD, 2>(st, st.area1, ai, P, wc, vc, idxC, &eaC, lane);
		errA = SubsetTable<kD, 3>(st, st.area1, ai, P, wa, va, idxA, &eaA, lane);
	}
	else if (MODE == 4)
	{
		int vc[8][4], va[4][4];
		Levels4<3>(epI, vc);
		Levels4<2>(epI, va);
		for (int k = 0; k < 8; k++)
			vc[k][a] = 0;
		for (int k = 0; k < 4; k++)
			for (int c = 0; c < 4; c++)
				if (c != a)
					va[k][c] = 0;
		errC = SubsetTable<kD, 3>(st, st.area1, ai, P, wc, vc, idxC, &eaC, lane);
		errA = SubsetTable<kD, 2>(st, st.area1, ai, P, wa, va, idxA, &eaA, lane);
	}
	else
	{
		int vc[4][4], va[4][4];
		Levels4<2>(epI, vc);
		Levels4<2>(epI, va);
		for (int k = 0; k < 4; k++)
		{
			vc[k][a] = 0;
			for (int c = 0; c < 4; c++)
				if (c != a)
					va[k][c] = 0;
		}
		errC = SubsetTable<kD, 2>(st, st.area1, ai, P, wc, vc, idxC, &eaC, lane);
		errA = SubsetTable<kD, 2>(st, st.area1, ai, P, wa, va, idxA, &eaA, lane);
	}
	R.errAlpha = (a == 0 ? eaA : eaC) * P.wA;
	R.errTotal = errC + errA;

	const int cb = idx32 ? 3 : 2;
	const int ab = (MODE == 4 && !idx32) ? 3 : 2;
	Ep mcolor = epS, malpha = epS;
	ReduceTable(0xFFFF, 0, cb, mcolor, idxC);
	ReduceTable(0xFFFF, 0, ab, malpha, idxA);
	const Ep ep = (mcolor & ~uint64_t(0xFFFF)) | (malpha & 0xFFFF);

	BitOut bw;
	if (MODE == 4)
	{
		bw.Put(16, 5);
		bw.Put(uint64_t(rotation & 3), 2);
		bw.Put(uint64_t((rotation >> 2) & 1), 1);
		const int order[3] = { 2, 1, 3 };
		for (int oc = 0; oc < 3; oc++)
			for (int k = 0; k < 2; k++)
				bw.Put(uint64_t(EpGet(ep, 2 * order[oc] + k) >> 3), 5);
		for (int k = 0; k < 2; k++)
			bw.Put(uint64_t(EpGet(ep, k) >> 2), 6);
		if (cb == 2)
		{
			bw.PutIndices(idxC, 2, 0, -1, -1);
			bw.PutIndices(idxA, 3, 0, -1, -1);
		}
		else
		{
			bw.PutIndices(idxA, 2, 0, -1, -1);
			bw.PutIndices(idxC, 3, 0, -1, -1);
		}
	}
	else
	{
		bw.Put(32, 6);
		bw.Put(uint64_t(rotation & 3), 2);
		const int order[3] = { 2, 1, 3 };
		for (int oc = 0; oc < 3; oc++)
			for (int k = 0; k < 2; k++)
				bw.Put(uint64_t(EpGet(ep, 2 * order[oc] + k) >> 1), 7);
		for (int k = 0; k < 2; k++)
			bw.Put(uint64_t(EpGet(ep, k)), 8);
		bw.PutIndices(idxC, 2, 0, -1, -1);
		bw.PutIndices(idxA, 2, 0, -1, -1);
	}
	lo = bw.lo;
	hi = bw.hi;
}

/* Final packing of modes 6 and 6Index2 (src/Bc7CoreMode6.cpp:933-1075,
   src/Bc7CoreMode6Index2.cpp:21-82). */
template<int kD, bool INDEX2>
__device__ void FinalPackMode6(WarpState& st, CellRegs& R, const Params& P, uint64_t& lo, uint64_t& hi, int lane)
{
	Ep ep = R.best[0];
	AreaInfo ai = R.a1;
	ai.zero = 0;
	const int w[4] = { P.wA, P.wG, P.wR, P.wB };
	uint64_t indices = 0;
	int ea = 0;
	if (INDEX2)
	{
		int vals[4][4];
		Levels4<2>(ep, vals);
		uint64_t idx2 = 0;
		R.errTotal = SubsetTable<kD, 2>(st, st.area1, ai, P, w, vals, idx2, &ea, lane);
		for (int i = 0; i < 16; i++)
		{
			uint64_t index = (idx2 >> (i << 1)) & 3u;
			index += index << 2;
			indices |= index << (i << 2);
		}
	}
	else
	{
		int vals[16][4];
		Levels4<4>(ep, vals);
		R.errTotal = SubsetTable<kD, 4>(st, st.area1, ai, P, w, vals, indices, &ea, lane);
	}
	R.errAlpha = ea * P.wA;
	if (indices & 8)
	{
		indices = ~indices;
		ep = EpSwapEnds(ep);
	}
	BitOut bw;
	bw.Put(64, 7);
	const int order[4] = { 2, 1, 3, 0 };
	for (int oc = 0; oc < 4; oc++)
		for (int k = 0; k < 2; k++)
			bw.Put(uint64_t(EpGet(ep, 2 * order[oc] + k) >> 1), 7);
	bw.Put(uint64_t(EpGet(ep, 0) & 1), 1);
	bw.Put(uint64_t(EpGet(ep, 1) & 1), 1);
	bw.PutIndices(indices, 4, 0, -1, -1);
	lo = bw.lo;
	hi = bw.hi;
}

template<int kD>
__device__ NEBC7_ONCE void FinalPack(WarpState& st, CellRegs& R, const Params& P, uint64_t& lo, uint64_t& hi, int lane)
{
	switch (R.bestMode)
	{
	case 0: FinalPackPartitioned<kD, 0>(st, R, P, lo, hi, lane); break;
	case 1: FinalPackPartitioned<kD, 1>(st, R, P, lo, hi, lane); break;
	case 2: FinalPackPartitioned<kD, 2>(st, R, P, lo, hi, lane); break;
	case 3: FinalPackPartitioned<kD, 3>(st, R, P, lo, hi, lane); break;
	case 4: FinalPackRot<kD, 4>(st, R, P, lo, hi, lane); break;
	case 5: FinalPackRot<kD, 5>(st, R, P, lo, hi, lane); break;
	case 6: FinalPackMode6<kD, false>(st, R, P, lo, hi, lane); break;
	case 7: FinalPackPartitioned<kD, 7>(st, R, P, lo, hi, lane); break;
	case 9: FinalPackMode6<kD, true>(st, R, P, lo, hi, lane); break;
	}
}

} // namespace nebc7
