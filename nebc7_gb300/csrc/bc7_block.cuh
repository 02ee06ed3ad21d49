/*
 * BC7 block encoder for sm_103a -- per-warp block state and block-level
 * primitives: BPTC decode / pack, block error and SSIM, pixel subsets
 * ("areas"), subset errors and the index selection with its SSIM
 * tie-break.
 *
 * One warp owns one 4x4 block.  Values that describe the block (errors,
 * best endpoints, flags) are warp-uniform registers; per-pixel data lives
 * in the warp's slice of shared memory.  Lanes 0..15 map to pixels where a
 * step is per pixel.  The semantics follow the reference block encoder
 * (src/Bc7Core.cpp, src/Metrics.cpp, src/Snippet*.h); each function cites
 * what it reproduces.
 */
#pragma once

#include "bc7_defs.cuh"

namespace nebc7 {

/* Endpoints of one subset: byte 2c = endpoint 0 of channel c, byte 2c + 1 =
   endpoint 1, channels A, G, R, B (the reference's packed __m128i form). */
typedef uint64_t Ep;

__device__ __forceinline__ int EpGet(Ep ep, int i) { return int((ep >> (8 * i)) & 0xFF); }
__device__ __forceinline__ Ep EpSetCh(Ep ep, int c, int color)
{
	const int s = 16 * c;
	return (ep & ~(uint64_t(0xFFFF) << s)) | (uint64_t(color & 0xFFFF) << s);
}
__device__ __forceinline__ Ep EpSwapEnds(Ep ep)
{
	/* swaps endpoint 0 and 1 of every channel */
	return ((ep & 0x00FF00FF00FF00FFull) << 8) | ((ep >> 8) & 0x00FF00FF00FF00FFull);
}
/* swaps channel 0 with the rotated channel (image order <-> block order) */
__device__ __forceinline__ Ep EpSwapRot(Ep ep, int rotation)
{
	const int a = RotChannel(rotation);
	if (!a)
		return ep;
	const uint64_t c0 = ep & 0xFFFF;
	const uint64_t ca = (ep >> (16 * a)) & 0xFFFF;
	ep &= ~(uint64_t(0xFFFF) | (uint64_t(0xFFFF) << (16 * a)));
	return ep | ca | (c0 << (16 * a));
}

/* A pixel subset in the order the reference builds it (src/Bc7Core.cpp:111):
   the subset's selection list (anchor first, then ascending pixel index) with
   the visible pixels first; transparent pixels carry zero data and an
   alpha-only mask. */
struct Area
{
	uint16_t px[16][4];
	uint16_t mk[16][4];
	uint8_t idx[16];
};

struct AreaInfo
{
	uint16_t minmax[8];
	uint16_t bounds[8];
	int count, active, zero;
	bool opaque;
};

struct __align__(16) WarpState
{
	uint8_t img[16][4];    /* source pixels, A,G,R,B */
	uint8_t msk[16][4];    /* mask bytes, A,G,R,B */
	uint16_t px[16][4];    /* masked data */
	uint16_t mk[16][4];    /* masks widened to 0 / 0xFFFF */
	uint8_t dec[16][4];    /* decoded block */
	Area area1;
	Area sub[3];
	int scan[64];
	int ways[16];
	int loops[16];
	int best[16];
};

/* Block-wide values shared by the mode encoders (the scalar part of the
   reference's Cell, src/Bc7Core.h:55). */
struct CellRegs
{
	Ep best[3];
	int bestParam;
	int bestMode;
	int opaqueAlphaError;
	int errAlpha, errTotal;
	int personalParam, personalMode;
	uint32_t visible;      /* bit i: pixel i has its G mask set */
	bool opaque;           /* every pixel's masked alpha is 255 */
	int denoiseStep;
	AreaInfo a1;
};

/* ---------------------------------------------------------------------- */
/* BPTC decode (src/Bc7Core.cpp:1446 and the ModeN::DecompressBlock)      */
/* ---------------------------------------------------------------------- */

struct Bits
{
	uint64_t lo, hi;
	int pos;

	__device__ int Get(int n)
	{
		uint64_t v;
		if (pos >= 64)
			v = hi >> (pos - 64);
		else if (pos + n <= 64)
			v = lo >> pos;
		else
			v = (lo >> pos) | (hi << (64 - pos));
		pos += n;
		return int(v & ((uint64_t(1) << n) - 1));
	}
};

__device__ __forceinline__ int Expand(int v, int bits)
{
	v <<= (8 - bits);
	return v | (v >> bits);
}

/* Reads the index of pixel `pix` from an index field starting at bit
   `start`: anchors carry one bit less. */
__device__ __forceinline__ int IndexAt(uint64_t lo, uint64_t hi, int start, int bits, int pix, int a0, int a1, int a2)
{
	int pos = start;
	for (int i = 0; i < pix; i++)
		pos += (i == a0 || i == a1 || i == a2) ? bits - 1 : bits;
	const int n = (pix == a0 || pix == a1 || pix == a2) ? bits - 1 : bits;
	uint64_t v;
	if (pos >= 64)
		v = hi >> (pos - 64);
	else if (pos + n <= 64)
		v = lo >> pos;
	else
		v = (lo >> pos) | (hi << (64 - pos));
	return int(v & ((uint64_t(1) << n) - 1));
}

/* Decodes the whole block: header into regs (best endpoints, parameter,
   mode) and pixel `pix` into out[4] (A,G,R,B).  Every lane can call it. */
__device__ inline void DecodeBlock(uint64_t lo, uint64_t hi, int pix, uint8_t out[4], Ep best[3], int& param, int& mode)
{
	const int encoded = int(lo & 0xFF);
	mode = 8;
	for (int m = 0; m < 8; m++)
		if (encoded & (1 << m))
		{
			mode = m;
			break;
		}
	best[0] = best[1] = best[2] = 0;
	param = 0;
	if (mode == 8)
	{
		out[0] = out[1] = out[2] = out[3] = 0;
		return;
	}
	Bits br{ lo, hi, mode + 1 };
	if (mode == 0 || mode == 1 || mode == 2 || mode == 3 || mode == 7)
	{
		const int ns = (mode == 0 || mode == 2) ? 3 : 2;
		const int partition = br.Get(mode == 0 ? 4 : 6);
		const int cbits = mode == 0 ? 4 : (mode == 1 ? 6 : (mode == 2 ? 5 : (mode == 3 ? 7 : 5)));
		const bool hasAlpha = mode == 7;
		const bool hasP = mode != 2;
		int e[3][2][4];
		const int order[3] = { 2, 1, 3 };
		for (int oc = 0; oc < 3; oc++)
			for (int s = 0; s < ns; s++)
				for (int k = 0; k < 2; k++)
					e[s][k][order[oc]] = br.Get(cbits);
		for (int s = 0; s < ns; s++)
			for (int k = 0; k < 2; k++)
				e[s][k][0] = hasAlpha ? br.Get(cbits) : 0;
		int p[3][2] = { { 0, 0 }, { 0, 0 }, { 0, 0 } };
		if (mode == 1)
		{
			for (int s = 0; s < ns; s++)
				p[s][0] = p[s][1] = br.Get(1);
		}
		else if (hasP)
		{
			for (int s = 0; s < ns; s++)
				for (int k = 0; k < 2; k++)
					p[s][k] = br.Get(1);
		}
		const int bits = cbits + (hasP ? 1 : 0);
		int ex[3][2][4];
		for (int s = 0; s < ns; s++)
			for (int k = 0; k < 2; k++)
				for (int c = 0; c < 4; c++)
				{
					if (c == 0 && !hasAlpha)
					{
						ex[s][k][c] = 255;
						continue;
					}
					int v = e[s][k][c];
					if (hasP)
						v = (v << 1) | p[s][k];
					ex[s][k][c] = Expand(v, bits);
				}
		const int ibits = (mode == 0 || mode == 1) ? 3 : 2;
		int a1, a2;
		if (ns == 3)
		{
			a1 = c_anchor23[partition];
			a2 = c_anchor33[partition];
		}
		else
		{
			a1 = c_anchor22[partition];
			a2 = -1;
		}
		const int idx = IndexAt(lo, hi, br.pos, ibits, pix, 0, a1, a2);
		const int* w = ibits == 3 ? c_interp3 : c_interp2;
		const int s = ns == 3 ? int((c_part3[partition] >> (2 * pix)) & 3) : int((c_part2[partition] >> (2 * pix)) & 3);
		for (int c = 0; c < 4; c++)
			out[c] = uint8_t(Interp(ex[s][0][c], ex[s][1][c], w[idx]));
		for (int si = 0; si < ns; si++)
		{
			Ep v = 0;
			for (int c = 0; c < 4; c++)
				v |= (uint64_t(ex[si][0][c]) << (16 * c)) | (uint64_t(ex[si][1][c]) << (16 * c + 8));
			best[si] = v;
		}
		param = partition;
		return;
	}
	if (mode == 4 || mode == 5)
	{
		const int rotation = br.Get(2);
		const int idxMode = mode == 4 ? br.Get(1) : 0;
		const int cbits = mode == 4 ? 5 : 7;
		const int abits = mode == 4 ? 6 : 8;
		int e[2][4];
		const int order[3] = { 2, 1, 3 };
		for (int oc = 0; oc < 3; oc++)
			for (int k = 0; k < 2; k++)
				e[k][order[oc]] = br.Get(cbits);
		for (int k = 0; k < 2; k++)
			e[k][0] = br.Get(abits);
		int ex[2][4];
		for (int k = 0; k < 2; k++)
		{
			for (int c = 1; c < 4; c++)
				ex[k][c] = Expand(e[k][c], cbits);
			ex[k][0] = Expand(e[k][0], abits);
		}
		const int startA = br.pos;
		const int startB = startA + (mode == 4 ? 31 : 31);
		const int idxA = IndexAt(lo, hi, startA, 2, pix, 0, -1, -1);
		const int idxB = IndexAt(lo, hi, startB, mode == 4 ? 3 : 2, pix, 0, -1, -1);
		int colorBits, alphaBits, ci, ai;
		if (mode == 4)
		{
			colorBits = idxMode ? 3 : 2;
			alphaBits = idxMode ? 2 : 3;
			ci = idxMode ? idxB : idxA;
			ai = idxMode ? idxA : idxB;
		}
		else
		{
			colorBits = alphaBits = 2;
			ci = idxA;
			ai = idxB;
		}
		const int* wc = InterpWeights(colorBits);
		const int* wa = InterpWeights(alphaBits);
		int v[4];
		v[0] = Interp(ex[0][0], ex[1][0], wa[ai]);
		for (int c = 1; c < 4; c++)
			v[c] = Interp(ex[0][c], ex[1][c], wc[ci]);
		const int a = RotChannel(rotation);
		if (a)
		{
			const int t = v[0];
			v[0] = v[a];
			v[a] = t;
		}
		for (int c = 0; c < 4; c++)
			out[c] = uint8_t(v[c]);
		Ep b = 0;
		for (int c = 0; c < 4; c++)
			b |= (uint64_t(ex[0][c]) << (16 * c)) | (uint64_t(ex[1][c]) << (16 * c + 8));
		best[0] = b;
		param = rotation | (idxMode << 2);
		return;
	}
	/* mode 6 */
	{
		int e[2][4];
		const int order[4] = { 2, 1, 3, 0 };
		for (int oc = 0; oc < 4; oc++)
			for (int k = 0; k < 2; k++)
				e[k][order[oc]] = br.Get(7);
		const int p0 = br.Get(1), p1 = br.Get(1);
		int ex[2][4];
		for (int c = 0; c < 4; c++)
		{
			ex[0][c] = (e[0][c] << 1) | p0;
			ex[1][c] = (e[1][c] << 1) | p1;
		}
		const int idx = IndexAt(lo, hi, br.pos, 4, pix, 0, -1, -1);
		for (int c = 0; c < 4; c++)
			out[c] = uint8_t(Interp(ex[0][c], ex[1][c], c_interp4[idx]));
		Ep b = 0;
		for (int c = 0; c < 4; c++)
			b |= (uint64_t(ex[0][c]) << (16 * c)) | (uint64_t(ex[1][c]) << (16 * c + 8));
		best[0] = b;
		param = 0;
	}
}

/* Warp: decodes the block into st.dec (lanes 0..15 one pixel each); returns
   the header in every lane. */
__device__ inline void DecodeToState(WarpState& st, uint64_t lo, uint64_t hi, Ep best[3], int& param, int& mode, int lane)
{
	uint8_t px[4];
	DecodeBlock(lo, hi, lane & 15, px, best, param, mode);
	if (lane < 16)
	{
		st.dec[lane][0] = px[0];
		st.dec[lane][1] = px[1];
		st.dec[lane][2] = px[2];
		st.dec[lane][3] = px[3];
	}
	__syncwarp();
}

/* ---------------------------------------------------------------------- */
/* Block error and SSIM (src/Metrics.cpp:7-151)                           */
/* ---------------------------------------------------------------------- */

template<int kD>
__device__ void CompareBlocks(const WarpState& st, const Params& P, int lane, int& alpha, int& total)
{
	unsigned s[4] = { 0, 0, 0, 0 };
	if (lane < 16)
	{
		for (int c = 0; c < 4; c++)
		{
			int q = Q<kD>(int(st.img[lane][c]) - int(st.dec[lane][c]));
			q &= int(st.mk[lane][c]);
			s[c] = unsigned(q * q);
		}
	}
	const int w[4] = { P.wA, P.wG, P.wR, P.wB };
	unsigned t = 0;
	unsigned a = 0;
	for (int c = 0; c < 4; c++)
	{
		const unsigned sum = __reduce_add_sync(kFull, s[c]) * unsigned(w[c]);
		if (c == 0)
			a = sum;
		t += sum;
	}
	alpha = int(a);
	total = int(t);
}

/* double arithmetic kept in the reference's operation order without
   contraction (the reference's SSE2 doubles have no FMA) */
__device__ __forceinline__ double SsimRatio(int sasb, int sab, int sasa_sbsb, int saa_sbb)
{
	const double k1 = (0.01 * 255 * 16) * (0.01 * 255 * 16);
	const double k2 = k1 * 9;
	const double num = __dmul_rn(__dadd_rn(double(sasb), k1), __dadd_rn(double(sab), k2));
	const double den = __dmul_rn(__dadd_rn(double(sasa_sbsb), k1), __dadd_rn(double(saa_sbb), k2));
	return __ddiv_rn(num, den);
}

__device__ inline void CompareBlocksSSIM(const WarpState& st, const Params& P, int lane, double& alpha, double& color)
{
	double r[4];
	for (int c = 0; c < 4; c++)
	{
		unsigned t = 0, s = 0;
		if (lane < 16)
		{
			const unsigned m = st.msk[lane][c];
			t = st.dec[lane][c] & m;
			s = st.img[lane][c] & m;
		}
		const unsigned sa = __reduce_add_sync(kFull, t);
		const unsigned sb = __reduce_add_sync(kFull, s);
		const unsigned sab = __reduce_add_sync(kFull, t * s);
		const unsigned saa_sbb = __reduce_add_sync(kFull, t * t + s * s);
		unsigned vab = sab << 5;
		unsigned vaa = saa_sbb << 4;
		unsigned sasb = sa * sb;
		sasb += sasb;
		const unsigned sasa_sbsb = sa * sa + sb * sb;
		vab -= sasb;
		vaa -= sasa_sbsb;
		r[c] = SsimRatio(int(sasb), int(vab), int(sasa_sbsb), int(vaa));
	}
	const double ssim = __dadd_rn(__dadd_rn(__dmul_rn(r[1], double(P.wG)), __dmul_rn(r[2], double(P.wR))), __dmul_rn(r[3], double(P.wB)));
	alpha = r[0];
	color = __ddiv_rn(ssim, double(P.wColor));
}

/* ---------------------------------------------------------------------- */
/* Areas (src/Bc7Core.cpp:111-492)                                        */
/* ---------------------------------------------------------------------- */

/* Data and mask of pixel i as an area sees it: visible pixels keep the
   cell data, transparent ones become zero data with an alpha-only mask. */
__device__ __forceinline__ void AreaPixel(const WarpState& st, const CellRegs& R, int i, int px[4], int mk[4])
{
	if ((R.visible >> i) & 1)
	{
		for (int c = 0; c < 4; c++)
		{
			px[c] = st.px[i][c];
			mk[c] = st.mk[i][c];
		}
	}
	else
	{
		for (int c = 0; c < 4; c++)
		{
			px[c] = 0;
			mk[c] = 0;
		}
		mk[0] = 0xFFFF;
	}
}

__device__ __forceinline__ void SwapPair(uint16_t* b, int lane)
{
	const uint16_t t = b[lane];
	b[lane] = b[lane + 1];
	b[lane + 1] = t;
}

/* Bounds, counts and channel orientation of the pixel subset `member`
   (bit i = pixel i); order-independent, so a lane can evaluate any subset. */
__device__ inline NEBC7_SHARED AreaInfo AreaStats(const WarpState& st, const CellRegs& R, const Params& P, uint32_t member)
{
	AreaInfo a;
	const uint32_t vis = member & R.visible;
	a.count = __popc(member);
	a.active = __popc(vis);
	a.zero = 0;  /* the caller knows the subset's anchor */

	int m0[4] = { 255, 255, 255, 255 }, m1[4] = { 0, 0, 0, 0 };
	int sum[4] = { 0, 0, 0, 0 };
	int sGR = 0, sRB = 0, sBG = 0, sAG = 0, sAR = 0, sAB = 0;
	const bool fast = (R.visible == 0xFFFF) && R.opaque;
	if (!fast && a.active < a.count)
		m0[0] = 0;
	for (int i = 0; i < 16; i++)
	{
		if (!((vis >> i) & 1))
			continue;
		const int v0 = st.px[i][0], v1 = st.px[i][1], v2 = st.px[i][2], v3 = st.px[i][3];
		const int v[4] = { v0, v1, v2, v3 };
		for (int c = 0; c < 4; c++)
		{
			m0[c] = min(m0[c], v[c]);
			m1[c] = max(m1[c], v[c]);
			sum[c] += v[c];
		}
		sGR += v1 * v2;
		sRB += v2 * v3;
		sBG += v3 * v1;
		sAG += v1 * v0;
		sAR += v2 * v0;
		sAB += v3 * v0;
	}
	if (!fast)
	{
		for (int c = 0; c < 4; c++)
			if (m1[c] < m0[c])
				m0[c] = 0;
	}
	uint16_t mb[8];
	for (int c = 0; c < 4; c++)
	{
		mb[2 * c] = uint16_t(m0[c]);
		mb[2 * c + 1] = uint16_t(m1[c]);
	}
	for (int k = 0; k < 8; k++)
		a.minmax[k] = mb[k];

	a.opaque = fast ? true : (mb[0] == 255);
	const long long n = a.active;
	if (a.opaque)
	{
		long long covGR = (long long)int(unsigned(sGR) * unsigned(n) - unsigned(sum[1]) * unsigned(sum[2]));
		long long covRB = (long long)int(unsigned(sRB) * unsigned(n) - unsigned(sum[2]) * unsigned(sum[3]));
		long long covBG = (long long)int(unsigned(sBG) * unsigned(n) - unsigned(sum[3]) * unsigned(sum[1]));
		if (covGR < 0)
		{
			SwapPair(mb, 4);
			covGR = -covGR;
			covRB = -covRB;
		}
		if (covBG < 0)
		{
			SwapPair(mb, 6);
			covBG = -covBG;
			covRB = -covRB;
		}
		if (!(covGR | covBG) && (covRB < 0))
		{
			SwapPair(mb, 6);
			covRB = -covRB;
		}
		for (int guard = 0; guard < 64; guard++)
		{
			bool changes = false;
			const long long b = covBG * P.wG + covRB * P.wR;
			if (b < 0)
			{
				SwapPair(mb, 6);
				covBG = -covBG;
				covRB = -covRB;
				changes = true;
			}
			const long long r = covGR * P.wG + covRB * P.wB;
			if (r < 0)
			{
				SwapPair(mb, 4);
				covGR = -covGR;
				covRB = -covRB;
				changes = true;
			}
			if (!changes)
				break;
		}
	}
	else
	{
		long long covGR = (long long)int(unsigned(sGR) * unsigned(n) - unsigned(sum[1]) * unsigned(sum[2]));
		long long covRB = (long long)int(unsigned(sRB) * unsigned(n) - unsigned(sum[2]) * unsigned(sum[3]));
		long long covBG = (long long)int(unsigned(sBG) * unsigned(n) - unsigned(sum[3]) * unsigned(sum[1]));
		long long covAG = (long long)int(unsigned(sAG) * unsigned(n) - unsigned(sum[1]) * unsigned(sum[0]));
		long long covAR = (long long)int(unsigned(sAR) * unsigned(n) - unsigned(sum[2]) * unsigned(sum[0]));
		long long covAB = (long long)int(unsigned(sAB) * unsigned(n) - unsigned(sum[3]) * unsigned(sum[0]));
		if (covAG < 0)
		{
			SwapPair(mb, 2);
			covAG = -covAG;
			covGR = -covGR;
			covBG = -covBG;
		}
		if (covAR < 0)
		{
			SwapPair(mb, 4);
			covAR = -covAR;
			covGR = -covGR;
			covRB = -covRB;
		}
		if (covAB < 0)
		{
			SwapPair(mb, 6);
			covAB = -covAB;
			covBG = -covBG;
			covRB = -covRB;
		}
		if (!covAR && (covGR < 0))
		{
			SwapPair(mb, 4);
			covGR = -covGR;
			covRB = -covRB;
		}
		if (!covAB && (covBG < 0))
		{
			SwapPair(mb, 6);
			covBG = -covBG;
			covRB = -covRB;
		}
		if (!(covAR | covAB | covGR | covBG) && (covRB < 0))
		{
			SwapPair(mb, 6);
			covRB = -covRB;
		}
		for (int guard = 0; guard < 64; guard++)
		{
			bool changes = false;
			const long long b = covAB * P.wA + covBG * P.wG + covRB * P.wR;
			if (b < 0)
			{
				SwapPair(mb, 6);
				covAB = -covAB;
				covBG = -covBG;
				covRB = -covRB;
				changes = true;
			}
			const long long r = covAR * P.wA + covGR * P.wG + covRB * P.wB;
			if (r < 0)
			{
				SwapPair(mb, 4);
				covAR = -covAR;
				covGR = -covGR;
				covRB = -covRB;
				changes = true;
			}
			const long long g = covAG * P.wA + covGR * P.wR + covBG * P.wB;
			if (g < 0)
			{
				SwapPair(mb, 2);
				covAG = -covAG;
				covGR = -covGR;
				covBG = -covBG;
				changes = true;
			}
			if (!changes)
				break;
		}
	}
	for (int k = 0; k < 8; k++)
		a.bounds[k] = mb[k];
	return a;
}

/* Writes the ordered pixel list of a subset into `ar` (lanes 0..15).
   `anchor` is the subset's first pixel; members follow in ascending order,
   visible pixels first. */
__device__ inline NEBC7_SHARED void BuildAreaList(Area& ar, const WarpState& st, const CellRegs& R, uint32_t member, int anchor, int lane)
{
	uint32_t rest = member & ~(1u << anchor);
	/* position of every member in the selection order */
	const uint32_t vis = member & R.visible;
	const uint32_t inv = member & ~R.visible;
	if (lane < 16 && ((member >> lane) & 1))
	{
		/* selection order: anchor, then ascending; rank within the list */
		int rankVis, pos;
		const bool isVis = (vis >> lane) & 1;
		const uint32_t group = isVis ? vis : inv;
		/* rank among the group in selection order */
		if (lane == anchor)
			rankVis = 0;
		else
			rankVis = (((group >> anchor) & 1) ? 1 : 0) + __popc(group & rest & ((1u << lane) - 1));
		pos = isVis ? rankVis : __popc(vis) + rankVis;
		ar.idx[pos] = uint8_t(lane);
		int px[4], mk[4];
		AreaPixel(st, R, lane, px, mk);
		for (int c = 0; c < 4; c++)
		{
			ar.px[pos][c] = uint16_t(px[c]);
			ar.mk[pos][c] = uint16_t(mk[c]);
		}
	}
	__syncwarp();
}

/* ---------------------------------------------------------------------- */
/* Subset errors                                                          */
/* ---------------------------------------------------------------------- */

/* Levels of one endpoint set: v[k] packs the four channels' interpolated
   values of level k in 16-bit lanes (A low). */
template<int BITS>
struct LevelSet
{
	int v[1 << BITS][4];

	__device__ __forceinline__ void Init(Ep ep)
	{
		const int* w = InterpWeights(BITS);
#pragma unroll
		for (int k = 0; k < (1 << BITS); k++)
#pragma unroll
			for (int c = 0; c < 4; c++)
				v[k][c] = Interp(EpGet(ep, 2 * c), EpGet(ep, 2 * c + 1), w[k]);
	}
};

/* Error of endpoints `ep` with a shared index over the visible pixels in
   `activeMask` (src/SnippetComputeOpaqueSubset2.h:7, 3.h:7,
   src/Bc7CoreMode6.cpp:130 and their Pair variants; channels with zero
   weight drop out).  Exact (no early exit): callers only compare it with
   thresholds, where the early-exit value decides the same way. */
template<int kD, int BITS>
__device__ int SubsetErrorMask(const WarpState& st, uint32_t activeMask, Ep ep, const int w[4])
{
	LevelSet<BITS> L;
	L.Init(ep);
	int sum = 0;
	for (int i = 0; i < 16; i++)
	{
		if (!((activeMask >> i) & 1))
			continue;
		const int p0 = st.px[i][0], p1 = st.px[i][1], p2 = st.px[i][2], p3 = st.px[i][3];
		int best = 0x7FFFFFFF;
#pragma unroll
		for (int k = 0; k < (1 << BITS); k++)
		{
			const int q0 = Q<kD>(p0 - L.v[k][0]), q1 = Q<kD>(p1 - L.v[k][1]);
			const int q2 = Q<kD>(p2 - L.v[k][2]), q3 = Q<kD>(p3 - L.v[k][3]);
			const int e = w[0] * q0 * q0 + w[1] * q1 * q1 + w[2] * q2 * q2 + w[3] * q3 * q3;
			best = min(best, e);
		}
		sum += best;
	}
	return sum;
}

/* Mode 4/5 error with separate color and alpha-slot indices
   (src/Bc7CoreMode4.cpp:159-839, src/Bc7CoreMode5.cpp:143-401): pixels are
   the Area1 view (transparent pixels with zero data and an alpha-only
   mask); mode 4 visits the visible pixels and adds (16 - active) times the
   alpha error of the lower alpha endpoint, mode 5 visits all 16.
   `epImg` in image channel order. */
template<int kD, int CB, int AB, bool MODE4>
__device__ int RotErrorExact(const WarpState& st, const CellRegs& R, Ep epImg, int rotation, const int w[4])
{
	const int a = RotChannel(rotation);
	LevelSet<CB> LC;
	LevelSet<AB> LA;
	LC.Init(epImg);
	LA.Init(epImg);
	int sum = 0;
	for (int i = 0; i < 16; i++)
	{
		const bool vis = (R.visible >> i) & 1;
		if (MODE4 && !vis)
			continue;
		int px[4], mk[4];
		AreaPixel(st, R, i, px, mk);
		int bestc = 0x7FFFFFFF;
#pragma unroll
		for (int k = 0; k < (1 << CB); k++)
		{
			int e = 0;
#pragma unroll
			for (int c = 0; c < 4; c++)
			{
				if (c == a)
					continue;
				const int q = Q<kD>(px[c] - LC.v[k][c]);
				e += w[c] * ((q * q) & mk[c]);
			}
			bestc = min(bestc, e);
		}
		int besta = 0x7FFFFFFF;
#pragma unroll
		for (int k = 0; k < (1 << AB); k++)
		{
			int pa = 0, va = 0, ma = 0;
#pragma unroll
			for (int c = 0; c < 4; c++)
				if (c == a)
				{
					pa = px[c];
					va = LA.v[k][c];
					ma = mk[c];
				}
			const int q = Q<kD>(pa - va);
			besta = min(besta, w[a] * ((q * q) & ma));
		}
		sum += besta + bestc;
	}
	if (MODE4 && R.a1.active < 16)
	{
		const int m = min(EpGet(epImg, 0), EpGet(epImg, 1));
		const int q = Q<kD>(m);
		sum += q * q * (w[0] * (16 - R.a1.active));
	}
	return sum;
}

/* (count - active) * wA * D(0, alpha)^2, alpha = endpoint pair of channel A,
   with the 2-bit table (src/Bc7CoreMode7.cpp:128) or the clamped 4-bit
   nibble table (src/Bc7CoreMode6.cpp:117). */
__device__ __forceinline__ int TransparentError2(const LevelTables& T, const Params& P, int count, int active, int alpha)
{
	int e = count - active;
	if (e)
	{
		e *= P.wA;
		const int v = DiffAt(T.d2v8, 0, alpha & 0xFF, (alpha >> 8) & 0xFF);
		e *= v * v;
	}
	return e;
}

__device__ __forceinline__ int TransparentError4(const LevelTables& T, const Params& P, int count, int active, int alpha)
{
	int e = count - active;
	if (e)
	{
		e *= P.wA;
		const int v = HalfAt(T.d4h, 0, alpha & 0xFF, (alpha >> 8) & 0xFF);
		e *= v * v;
	}
	return e;
}

/* ---------------------------------------------------------------------- */
/* Index selection with the SSIM tie-break (src/Bc7Core.cpp:746-1429)     */
/* ---------------------------------------------------------------------- */

/* vals: M levels of the four channels (A,G,R,B), possibly channel-masked.
   Writes the chosen index of every area position to st.best[] and returns
   the quantised error.  Warp-collective. */
template<int kD, int M>
__device__ int ComputeSubsetTable(WarpState& st, const Area& ar, const AreaInfo& ai, const Params& P, const int w[4], const int vals[M][4], int lane)
{
	const int denoiseStep = P.denoiseStep * (ai.opaque ? P.wColor : P.wColorAlpha);

	auto same = [&](int i, int j) -> bool {
		return vals[i][0] == vals[j][0] && vals[i][1] == vals[j][1] && vals[i][2] == vals[j][2] && vals[i][3] == vals[j][3];
	};
	int good = 1;
	{
		const int m = M >> 1;
		for (int i = 1; i < m; i++)
			good |= int(!same(i - 1, i)) << i;
		for (int i = m; i < M - 1; i++)
			good |= int(!same(i, i + 1)) << i;
		good |= int(!same(0, M - 1)) << (M - 1);
		good &= ~(int(same(m - 1, m)) << m);
	}

	unsigned bottomHi = 0;
	if (lane < ai.active)
	{
		int p[4];
		for (int c = 0; c < 4; c++)
			p[c] = ar.px[lane][c];
		uint64_t bottom = ~uint64_t(0);
		uint64_t keys[M];
#pragma unroll
		for (int k = 0; k < M; k++)
		{
			int hi = 0, lo = 0;
#pragma unroll
			for (int c = 0; c < 4; c++)
			{
				const int d = vals[k][c] - p[c];
				const int q = Q<kD>(d);
				hi += w[c] * q * q;
				lo += w[c] * int(int16_t(uint16_t((d * d) & 0xFFFF) ^ 0x8000));
			}
			keys[k] = (uint64_t(unsigned(hi)) << 32) | uint64_t(unsigned(lo));
			bottom = keys[k] < bottom ? keys[k] : bottom;
		}
		int way = 0;
#pragma unroll
		for (int k = 0; k < M; k++)
			way |= int(keys[k] == bottom) << k;
		bottomHi = unsigned(bottom >> 32);
		way &= good;
		const int kk = way & -way;
		way = (int(bottomHi << (kD + kD)) <= denoiseStep) ? kk : way;
		st.ways[lane] = (way != kk) ? way | (1 << M) : 0;
		st.loops[lane] = __popc(unsigned(kk - 1));
	}
	int errorBlock = int(__reduce_add_sync(kFull, bottomHi));

	if (ai.active < ai.count)
	{
		const int alpha0 = vals[0][0];
		const int alpha1 = vals[M - 1][0];
		int bottom = alpha1 < alpha0 ? alpha1 : alpha0;
		const int index = (bottom != alpha0) ? M - 1 : 0;
		if (!kD)
			bottom = bottom > 0x7F ? 0x7F : bottom;
		else
			bottom >>= kD;
		errorBlock += bottom * bottom * w[0] * (ai.count - ai.active);
		if (lane >= ai.active && lane < ai.count)
		{
			st.ways[lane] = 0;
			st.loops[lane] = index;
		}
	}
	if (lane >= ai.count && lane < 16)
	{
		st.ways[lane] = 0;
		st.loops[lane] = 0;
	}
	__syncwarp();

	const bool any = __any_sync(kFull, lane < 16 && st.ways[lane] > 0);
	if (!any)
	{
		if (lane < 16)
			st.best[lane] = st.loops[lane];
		__syncwarp();
		return errorBlock;
	}

	/* enumerate every combination of tied indices in the reference's odometer
	   order (pixel 0 the fastest digit, each digit over its tied indices in
	   ascending order) and keep the first maximum of the weighted SSIM
	   (src/Bc7Core.cpp:1341-1428).  Lane j evaluates combination base + j
	   on its own, so 32 combinations are in flight; the chunk's maximum and
	   its first lane then meet the running best with the reference's strict
	   comparison, which keeps the first maximum in odometer order.  At most
	   2^20 combinations are visited. */
	double bestSsim = -(double(P.wColorAlpha) + 0.1);
	const int count = ai.count;
	const int active = ai.active;
	const int shift = count > 8 ? 4 : (count > 4 ? 3 : (count > 2 ? 2 : (count > 1 ? 1 : 0)));
	int total = 1;
	for (int i = 0; i < active; i++)
	{
		const int way = st.ways[i];
		const int n = way ? __popc(unsigned(way) & ((1u << M) - 1)) : 1;
		total = (total > (1 << 20) / n) ? (1 << 20) + 1 : total * n;
	}
	if (total > (1 << 20))
		total = 1 << 20;
	int bestN = 0;
	for (int base = 0; base < total; base += 32)
	{
		const int n0 = base + lane;
		double ssim = -(double(P.wColorAlpha) + 0.1);
		if (n0 < total)
		{
			/* the digits of combination n0: each tied pixel's index */
			int idx[16];
			int rest = n0;
			for (int i = 0; i < 16; i++)
			{
				const int way = st.ways[i];
				int k = st.loops[i];
				if (i < active && way)
				{
					const unsigned tied = unsigned(way) & ((1u << M) - 1);
					const int n = __popc(tied);
					int d = rest % n;
					rest /= n;
					unsigned t = tied;
					while (d-- > 0)
						t &= t - 1;
					k = __ffs(t) - 1;
				}
				idx[i] = k;
			}
			for (int c = 0; c < 4; c++)
			{
				unsigned sa = 0, sb = 0, sab = 0, saa_sbb = 0;
				for (int i = 0; i < count; i++)
				{
					const unsigned t = unsigned(vals[idx[i]][c] & ar.mk[i][c]);
					const unsigned b = unsigned(ar.px[i][c]);
					sa += t;
					sb += b;
					sab += (t * b) & 0xFFFF;
					saa_sbb += ((t * t) & 0xFFFF) + ((b * b) & 0xFFFF);
				}
				unsigned vab = sab << (shift + 1);
				unsigned vaa = saa_sbb << shift;
				unsigned sasb = sa * sb;
				sasb += sasb;
				const unsigned sasa_sbsb = sa * sa + sb * sb;
				vab -= sasb;
				vaa -= sasa_sbsb;
				const double r = SsimRatio(int(sasb), int(vab), int(sasa_sbsb), int(vaa));
				ssim = (c == 0) ? __dmul_rn(r, double(w[0])) : __dadd_rn(ssim, __dmul_rn(r, double(w[c])));
			}
		}
		/* the chunk's maximum (exact comparisons of doubles) and its first lane */
		double m = ssim;
		for (int o = 16; o > 0; o >>= 1)
		{
			const double v = __shfl_xor_sync(kFull, m, o);
			m = v > m ? v : m;
		}
		const unsigned at = __ballot_sync(kFull, n0 < total && ssim == m);
		if (bestSsim < m)
		{
			bestSsim = m;
			bestN = base + __ffs(at) - 1;
		}
	}
	/* the indices of the winning combination */
	if (lane < 16)
	{
		int k = st.loops[lane];
		int rest = bestN;
		for (int i = 0; i < 16; i++)
		{
			const int way = st.ways[i];
			if (i < active && way)
			{
				const unsigned tied = unsigned(way) & ((1u << M) - 1);
				const int n = __popc(tied);
				const int d = rest % n;
				rest /= n;
				if (i == lane)
				{
					unsigned t = tied;
					for (int e = 0; e < d; e++)
						t &= t - 1;
					k = __ffs(t) - 1;
				}
			}
		}
		st.best[lane] = k;
	}
	__syncwarp();
	return errorBlock;
}

} // namespace nebc7
