/*
 * CPU oracle for the BC7 block encoder -- block state, metrics and search
 * primitives (test infrastructure only; see port_tables.h).  Scalar
 * restatement of reference src/Bc7Core.cpp:24-1444, src/Metrics.cpp and
 * src/Snippet*.h; each function cites the lines it follows.  Where the
 * reference relies on x86 integer behaviour (wrapping adds, shift counts
 * taken modulo 32, cvttps of NaN), the same behaviour is spelled out.
 */
#include "port_core.h"
#include "port_counters.h"

#include <algorithm>
#include <string.h>
#include <math.h>

namespace nebc7_oracle {

static bool gPca = false;

void SetPca(bool on)
{
	gPca = on;
}

void MakeConfig(Config& cfg, int denoise, int denoiseStep, bool doDraft, bool doNormal, bool doSlow, bool linearData)
{
	cfg.pca = gPca;
	cfg.denoise = denoise;
	cfg.denoiseStep = denoiseStep;
	cfg.doDraft = doDraft;
	cfg.mode6Index2Only = false;
	cfg.doNormal = doNormal;
	cfg.doSlow = doSlow;
	/* src/Bc7Tables.cpp:789-808 */
	if (linearData)
	{
		cfg.wA = cfg.wG = cfg.wR = cfg.wB = 1;
	}
	else
	{
		cfg.wA = 1000;
		cfg.wG = 715;
		cfg.wR = 213;
		cfg.wB = 72;
	}
	cfg.wColor = cfg.wG + cfg.wR + cfg.wB;
	cfg.wColorAlpha = cfg.wColor + cfg.wA;
	cfg.lt = &GetLevelTables(denoise);
	cfg.sel = &GetSelection();
}

void LevelsInit(Levels& L, const Config& cfg)
{
	L.minErr = cfg.MaxColorAlphaError();
	L.count = 0;
}

/* ---------------------------------------------------------------------- */
/* Area construction, src/Bc7Core.cpp:111-492                             */
/* ---------------------------------------------------------------------- */

static inline void SwapLanes(uint16_t* b, int lane)
{
	uint16_t t = b[lane];
	b[lane] = b[lane + 1];
	b[lane + 1] = t;
}

void MakeAreaFromCell(const Config& cfg, Area& area, const Cell& cell, int count, uint64_t indices)
{
	area.count = uint32_t(count);
	area.zero = uint8_t(indices & 0xF);

	int m0[8], m1[8];
	for (int k = 0; k < 8; k++)
	{
		m0[k] = 255;
		m1[k] = 0;
	}

	uint32_t active;
	const uint32_t flags = uint32_t(cell.visibleFlags);
	if (flags == 0xFFFF)
	{
		for (int i = 0; i < 16; i++)
			area.idx[i] = uint8_t((indices >> (4 * i)) & 0xF);
		active = uint32_t(count);

		if (cell.opaque)
		{
			/* all-visible opaque fast path, :137-239 */
			area.active = active;
			int64_t sum[4] = { 0, 0, 0, 0 };
			int64_t sGR = 0, sRB = 0, sBG = 0;
			for (uint32_t i = 0; i < active; i++)
			{
				const int index = area.idx[i];
				for (int c = 0; c < 4; c++)
				{
					area.px[i][c] = cell.px[index][c];
					area.mk[i][c] = cell.mk[index][c];
					int v = int16_t(cell.px[index][c]);
					int m = int16_t(cell.mk[index][c]);
					m0[c] = std::min(m0[c], v);
					m1[c] = std::max(m1[c], v);
					m0[4 + c] = std::min(m0[4 + c], m);
					m1[4 + c] = std::max(m1[4 + c], m);
					sum[c] += v;
				}
				const int g = cell.px[index][1], r = cell.px[index][2], b = cell.px[index][3];
				sGR += g * r;
				sRB += r * b;
				sBG += b * g;
			}
			uint16_t mb[8];
			for (int c = 0; c < 4; c++)
			{
				mb[2 * c] = uint16_t(m0[c]);
				mb[2 * c + 1] = uint16_t(m1[c]);
			}
			memcpy(area.minmax, mb, sizeof(mb));
			area.opaque = true;

			const int64_t n = active;
			int64_t covGR = int32_t(int32_t(sGR) * int32_t(n) - int32_t(sum[1]) * int32_t(sum[2]));
			int64_t covRB = int32_t(int32_t(sRB) * int32_t(n) - int32_t(sum[2]) * int32_t(sum[3]));
			int64_t covBG = int32_t(int32_t(sBG) * int32_t(n) - int32_t(sum[3]) * int32_t(sum[1]));

			if (covGR < 0)
			{
				SwapLanes(mb, 4);
				covGR = -covGR;
				covRB = -covRB;
			}
			if (covBG < 0)
			{
				SwapLanes(mb, 6);
				covBG = -covBG;
				covRB = -covRB;
			}
			if (!(covGR | covBG) && (covRB < 0))
			{
				SwapLanes(mb, 6);
				covRB = -covRB;
			}
			for (;;)
			{
				bool changes = false;
				int64_t b = covBG * cfg.wG + covRB * cfg.wR;
				if (b < 0)
				{
					SwapLanes(mb, 6);
					covBG = -covBG;
					covRB = -covRB;
					changes = true;
				}
				int64_t r = covGR * cfg.wG + covRB * cfg.wB;
				if (r < 0)
				{
					SwapLanes(mb, 4);
					covGR = -covGR;
					covRB = -covRB;
					changes = true;
				}
				if (!changes)
					break;
			}
			memcpy(area.bounds, mb, sizeof(mb));
			return;
		}
	}
	else
	{
		/* visible pixels first, then the transparent ones, :241-278 */
		uint8_t transparent[16];
		int nv = 0, nt = 0;
		for (int i = 0; i < count; i++)
		{
			const int index = int(indices & 0xF);
			indices >>= 4;
			if ((flags >> index) & 1)
				area.idx[nv++] = uint8_t(index);
			else
				transparent[nt++] = uint8_t(index);
		}
		active = uint32_t(nv);
		if (active < uint32_t(count))
		{
			m0[0] = 0;
			for (int k = 0; k < nt; k++)
			{
				area.idx[nv + k] = transparent[k];
				for (int c = 0; c < 4; c++)
				{
					area.px[nv + k][c] = 0;
					area.mk[nv + k][c] = 0;
				}
				area.mk[nv + k][0] = 0xFFFF;
			}
		}
	}

	area.active = active;

	/* :284-304 */
	int64_t sum[4] = { 0, 0, 0, 0 };
	int64_t sGR = 0, sRB = 0, sBG = 0, sAG = 0, sAR = 0, sAB = 0;
	for (uint32_t i = 0; i < active; i++)
	{
		const int index = area.idx[i];
		for (int c = 0; c < 4; c++)
		{
			area.px[i][c] = cell.px[index][c];
			area.mk[i][c] = cell.mk[index][c];
			int v = int16_t(cell.px[index][c]);
			int m = int16_t(cell.mk[index][c]);
			m0[c] = std::min(m0[c], v);
			m1[c] = std::max(m1[c], v);
			m0[4 + c] = std::min(m0[4 + c], m);
			m1[4 + c] = std::max(m1[4 + c], m);
			sum[c] += v;
		}
		const int a = cell.px[index][0], g = cell.px[index][1], r = cell.px[index][2], b = cell.px[index][3];
		sGR += g * r;
		sRB += r * b;
		sBG += b * g;
		sAG += g * a;
		sAR += r * a;
		sAB += b * a;
	}

	/* :306 min := 0 where max < min */
	for (int k = 0; k < 8; k++)
	{
		if (m1[k] < m0[k])
			m0[k] = 0;
	}
	uint16_t mb[8];
	for (int c = 0; c < 4; c++)
	{
		mb[2 * c] = uint16_t(m0[c]);
		mb[2 * c + 1] = uint16_t(m1[c]);
	}
	memcpy(area.minmax, mb, sizeof(mb));

	area.opaque = (mb[0] == 255);

	const int32_t n = int32_t(active);
	if (area.opaque)
	{
		/* :322-382 */
		int64_t covGR = int32_t(int32_t(sGR) * n - int32_t(sum[1]) * int32_t(sum[2]));
		int64_t covRB = int32_t(int32_t(sRB) * n - int32_t(sum[2]) * int32_t(sum[3]));
		int64_t covBG = int32_t(int32_t(sBG) * n - int32_t(sum[3]) * int32_t(sum[1]));

		if (covGR < 0)
		{
			SwapLanes(mb, 4);
			covGR = -covGR;
			covRB = -covRB;
		}
		if (covBG < 0)
		{
			SwapLanes(mb, 6);
			covBG = -covBG;
			covRB = -covRB;
		}
		if (!(covGR | covBG) && (covRB < 0))
		{
			SwapLanes(mb, 6);
			covRB = -covRB;
		}
		for (;;)
		{
			bool changes = false;
			int64_t b = covBG * cfg.wG + covRB * cfg.wR;
			if (b < 0)
			{
				SwapLanes(mb, 6);
				covBG = -covBG;
				covRB = -covRB;
				changes = true;
			}
			int64_t r = covGR * cfg.wG + covRB * cfg.wB;
			if (r < 0)
			{
				SwapLanes(mb, 4);
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
		/* :383-489 */
		int64_t covGR = int32_t(int32_t(sGR) * n - int32_t(sum[1]) * int32_t(sum[2]));
		int64_t covRB = int32_t(int32_t(sRB) * n - int32_t(sum[2]) * int32_t(sum[3]));
		int64_t covBG = int32_t(int32_t(sBG) * n - int32_t(sum[3]) * int32_t(sum[1]));
		int64_t covAG = int32_t(int32_t(sAG) * n - int32_t(sum[1]) * int32_t(sum[0]));
		int64_t covAR = int32_t(int32_t(sAR) * n - int32_t(sum[2]) * int32_t(sum[0]));
		int64_t covAB = int32_t(int32_t(sAB) * n - int32_t(sum[3]) * int32_t(sum[0]));

		if (covAG < 0)
		{
			SwapLanes(mb, 2);
			covAG = -covAG;
			covGR = -covGR;
			covBG = -covBG;
		}
		if (covAR < 0)
		{
			SwapLanes(mb, 4);
			covAR = -covAR;
			covGR = -covGR;
			covRB = -covRB;
		}
		if (covAB < 0)
		{
			SwapLanes(mb, 6);
			covAB = -covAB;
			covBG = -covBG;
			covRB = -covRB;
		}
		if (!covAR && (covGR < 0))
		{
			SwapLanes(mb, 4);
			covGR = -covGR;
			covRB = -covRB;
		}
		if (!covAB && (covBG < 0))
		{
			SwapLanes(mb, 6);
			covBG = -covBG;
			covRB = -covRB;
		}
		if (!(covAR | covAB | covGR | covBG) && (covRB < 0))
		{
			SwapLanes(mb, 6);
			covRB = -covRB;
		}
		for (;;)
		{
			bool changes = false;
			int64_t b = covAB * cfg.wA + covBG * cfg.wG + covRB * cfg.wR;
			if (b < 0)
			{
				SwapLanes(mb, 6);
				covAB = -covAB;
				covBG = -covBG;
				covRB = -covRB;
				changes = true;
			}
			int64_t r = covAR * cfg.wA + covGR * cfg.wG + covRB * cfg.wB;
			if (r < 0)
			{
				SwapLanes(mb, 4);
				covAR = -covAR;
				covGR = -covGR;
				covRB = -covRB;
				changes = true;
			}
			int64_t g = covAG * cfg.wA + covGR * cfg.wR + covBG * cfg.wB;
			if (g < 0)
			{
				SwapLanes(mb, 2);
				covAG = -covAG;
				covGR = -covGR;
				covBG = -covBG;
				changes = true;
			}
			if (!changes)
				break;
		}
	}
	memcpy(area.bounds, mb, sizeof(mb));
}

Area& GetArea(const Config& cfg, Area& area, bool& lazy, const Cell& cell, uint64_t indices)
{
	/* src/Bc7Core.h:123 */
	if (lazy)
	{
		lazy = false;
		MakeAreaFromCell(cfg, area, cell, int(indices & 0xF), indices >> 4);
	}
	return area;
}

/* ---------------------------------------------------------------------- */
/* Interpolation and errors                                               */
/* ---------------------------------------------------------------------- */

static inline int Saturate8(int v)
{
	return v < 0 ? 0 : (v > 255 ? 255 : v);
}

void PackEndpoints(const V8& mc, uint8_t ep[8])
{
	/* _mm_packus_epi16: signed 16-bit to unsigned 8-bit with saturation */
	for (int i = 0; i < 8; i++)
		ep[i] = uint8_t(Saturate8(mc.l[i]));
}

static inline const int* WeightsFor(int indexBits)
{
	return indexBits == 2 ? kInterp2 : (indexBits == 3 ? kInterp3 : kInterp4);
}

void InterpolateLevels(const uint8_t ep[8], int indexBits, uint16_t vals[16][4])
{
	const int* w = WeightsFor(indexBits);
	const int levels = 1 << indexBits;
	for (int k = 0; k < levels; k++)
		for (int c = 0; c < 4; c++)
			vals[k][c] = uint16_t((ep[2 * c] * (64 - w[k]) + ep[2 * c + 1] * w[k] + 32) >> 6);
}

int SubsetError(const Config& cfg, const Area& area, const uint8_t ep[8], int indexBits, const int w[4], int water)
{
	uint16_t vals[16][4];
	InterpolateLevels(ep, indexBits, vals);
	const int levels = 1 << indexBits;

	int sum = 0;
	uint32_t i = 0;
	for (; i < area.active; i++)
	{
		int best = 0x7FFFFFFF;
		for (int k = 0; k < levels; k++)
		{
			int e = 0;
			for (int c = 0; c < 4; c++)
			{
				const int q = cfg.Q(int(area.px[i][c]) - int(vals[k][c]));
				e += w[c] * q * q;
			}
			best = e < best ? e : best;
		}
		sum += best;
		if (!(water > sum))
		{
			i++;
			break;
		}
	}
	PORT_COUNT(kErrCalls, 1);
	PORT_COUNT(kErrTerms, uint64_t(i) * levels * ((w[0] != 0) + (w[1] != 0) + (w[2] != 0) + (w[3] != 0)));
	return sum;
}

/* src/Bc7Core.cpp:746-1429 */
int ComputeSubsetTable(const Config& cfg, const Area& area, const int w[4], int M, const uint16_t vals[16][4], int best[16])
{
	const int denoiseStep = cfg.denoiseStep * (area.opaque ? cfg.wColor : cfg.wColorAlpha);

	auto v64 = [&](int k) -> uint64_t {
		return uint64_t(vals[k][0]) | (uint64_t(vals[k][1]) << 16) | (uint64_t(vals[k][2]) << 32) | (uint64_t(vals[k][3]) << 48);
	};

	int good = 1;
	{
		const int m = M >> 1;
		for (int i = 1; i < m; i++)
			good |= int(v64(i - 1) != v64(i)) << i;
		for (int i = m; i < M - 1; i++)
			good |= int(v64(i) != v64(i + 1)) << i;
		good |= int(v64(0) != v64(M - 1)) << (M - 1);
		good &= ~(int(v64(m - 1) == v64(m)) << m);
	}

	int ways[16], loops[16];
	int errorBlock = 0;

	for (uint32_t i = 0; i < area.active; i++)
	{
		uint64_t keys[16];
		uint64_t bottom = ~uint64_t(0);
		for (int k = 0; k < M; k++)
		{
			int32_t hi = 0, lo = 0;
			for (int c = 0; c < 4; c++)
			{
				const int d = int(vals[k][c]) - int(area.px[i][c]);
				const int q = cfg.Q(d);
				hi += w[c] * q * q;
				const int16_t sq = int16_t(uint16_t((d * d) & 0xFFFF) ^ 0x8000);
				lo += w[c] * sq;
			}
			keys[k] = (uint64_t(uint32_t(hi)) << 32) | uint64_t(uint32_t(lo));
			bottom = keys[k] < bottom ? keys[k] : bottom;
		}
		int way = 0;
		for (int k = 0; k < M; k++)
			way |= int(keys[k] == bottom) << k;

		bottom >>= 32;
		errorBlock += int(bottom);

		way &= good;
		int k = way & -way;
		way = (int(uint32_t(bottom) << (cfg.denoise + cfg.denoise)) <= denoiseStep) ? k : way;
		ways[i] = (way != k) ? way | (1 << M) : 0;
		int loop = 0;
		for (uint32_t t = uint32_t(k - 1); t; t &= t - 1)
			loop++;
		loops[i] = loop;
	}

	if (area.active < area.count)
	{
		const int alpha0 = vals[0][0];
		const int alpha1 = vals[M - 1][0];
		int bottom = (alpha1 < alpha0) ? alpha1 : alpha0;
		const int index = (bottom != alpha0) ? M - 1 : 0;
		if (!cfg.denoise)
			bottom = (bottom > 0x7F) ? 0x7F : bottom;
		else
			bottom >>= cfg.denoise;
		errorBlock += bottom * bottom * w[0] * int(area.count - area.active);
		for (uint32_t i = area.active; i < area.count; i++)
		{
			ways[i] = 0;
			loops[i] = index;
		}
	}

	for (uint32_t i = area.count; i < 16; i++)
		ways[i] = 0;

	{
		bool any = false;
		for (int i = 0; i < 16; i++)
			any |= ways[i] > 0;
		if (!any)
		{
			for (int i = 0; i < 16; i++)
				best[i] = loops[i];
			return errorBlock;
		}
	}

	/* SSIM tie-break over all tied index combinations, :1341-1428 */
	const double k1 = (0.01 * 255 * 16) * (0.01 * 255 * 16);
	const double k2 = k1 * 9;
	double bestSsim = -(cfg.wColorAlpha + 0.1);

	const int count = int(area.count);
	int shift;
	if (count > 8)
		shift = 4;
	else if (count > 4)
		shift = 3;
	else if (count > 2)
		shift = 2;
	else if (count > 1)
		shift = 1;
	else
		shift = 0;

	for (;;)
	{
		int32_t sa[4] = { 0, 0, 0, 0 }, sb[4] = { 0, 0, 0, 0 }, sab[4] = { 0, 0, 0, 0 }, saa_sbb[4] = { 0, 0, 0, 0 };
		for (int i = 0; i < count; i++)
		{
			for (int c = 0; c < 4; c++)
			{
				const int32_t b = area.px[i][c];
				const int32_t t = vals[loops[i]][c] & area.mk[i][c];
				sa[c] += t;
				sb[c] += b;
				sab[c] += int32_t(uint16_t(t * b));
				saa_sbb[c] += int32_t(uint16_t(t * t)) + int32_t(uint16_t(b * b));
			}
		}
		double ssim = 0;
		for (int c = 0; c < 4; c++)
		{
			int32_t vab = int32_t(uint32_t(sab[c]) << (shift + 1));
			int32_t vaa = int32_t(uint32_t(saa_sbb[c]) << shift);
			int32_t sasb = int32_t(uint32_t(sa[c]) * uint32_t(sb[c]));
			sasb = int32_t(uint32_t(sasb) + uint32_t(sasb));
			int32_t sasa_sbsb = int32_t(uint32_t(sa[c]) * uint32_t(sa[c]) + uint32_t(sb[c]) * uint32_t(sb[c]));
			vab = int32_t(uint32_t(vab) - uint32_t(sasb));
			vaa = int32_t(uint32_t(vaa) - uint32_t(sasa_sbsb));
			const double num = (double(sasb) + k1) * (double(vab) + k2);
			const double den = (double(sasa_sbsb) + k1) * (double(vaa) + k2);
			const double s = num / den;
			if (c == 0)
				ssim = s * double(w[0]);
			else
				ssim += s * double(w[c]);
		}

		if (bestSsim < ssim)
		{
			bestSsim = ssim;
			for (int i = 0; i < 16; i++)
				best[i] = loops[i];
		}

		int i = 0;
		for (;;)
		{
			if (int way = ways[i])
			{
				int k = loops[i];
				do
				{
					k++;
				} while ((way & (1 << k)) == 0);
				if (k < M)
				{
					loops[i] = k;
					break;
				}
				k = 0;
				while ((way & (1 << k)) == 0)
					k++;
				loops[i] = k;
			}
			if (++i >= int(area.active))
				return errorBlock;
		}
	}
}

/* ---------------------------------------------------------------------- */
/* Candidate enumeration                                                  */
/* ---------------------------------------------------------------------- */

/* x86 32-bit integer behaviour the reference's window arithmetic relies on. */
static inline int32_t Wadd(int32_t a, int32_t b) { return int32_t(uint32_t(a) + uint32_t(b)); }
static inline int32_t Wsub(int32_t a, int32_t b) { return int32_t(uint32_t(a) - uint32_t(b)); }
static inline int32_t Wmul(int32_t a, int32_t b) { return int32_t(uint32_t(a) * uint32_t(b)); }
static inline int32_t Sar(int32_t a, int s) { return a >> s; /* arithmetic on every target this builds for */ }
static inline uint32_t Shr32(uint32_t v, uint32_t s) { return v >> (s & 31); }

/* d = floor(sqrt(top - 1)) as the reference computes it
   (src/SnippetLevelsBuffer.h:78-88): _mm_cvttps_epi32 of a correctly
   rounded single-precision square root, NaN (negative top) giving INT_MIN. */
static int32_t WindowRadius(const Config& cfg, int32_t top)
{
	int32_t d;
	if (top < 0)
	{
		d = INT32_MIN;
	}
	else
	{
		const float f = sqrtf(float(top));
		d = f >= 2147483648.0f ? INT32_MIN : int32_t(f);
	}
	d = Wsub(d, int32_t(Wmul(d, d) >= top));
	if (cfg.denoise)
	{
		d = int32_t(uint32_t(d) << cfg.denoise);
		d = Wadd(d, (1 << cfg.denoise) - 1);
	}
	return d;
}

struct Window
{
	int32_t LH, HL, HH;
};

/* src/SnippetLevelsBuffer.h:122-132 */
static Window MakeWindow(int32_t L, int32_t H, int32_t d, int bits, int shift)
{
	const int32_t tailmask = (1 << (8 - bits)) - 1;
	int32_t LH = std::min(Wadd(L, d), int32_t(255));
	int32_t HL = std::max(Wsub(H, d), int32_t(0));
	LH = std::min(Wadd(Wsub(H, Sar(H, shift)), tailmask), Wsub(LH, Sar(LH, shift))) & ~tailmask;
	HL = std::max(Wsub(L, Sar(L, shift)), Wadd(Wsub(HL, Sar(HL, shift)), tailmask)) & ~tailmask;
	Window w;
	w.LH = Sar(LH, 8 - shift);
	w.HL = Sar(HL, 8 - shift);
	w.HH = 0x100 >> (8 - shift);
	return w;
}

static inline int DecodeColor(uint32_t c, int shift, bool reverse)
{
	int cc = int(c);
	if (reverse)
	{
		int cL = (cc >> shift) << (8 - shift);
		int cH = (cc & ((1 << shift) - 1)) << (8 - shift);
		return ((cH + (cH >> shift)) << 8) + cL + (cL >> shift);
	}
	if (shift != 8)
	{
		int cH = (cc >> shift) << (8 - shift);
		int cL = (cc & ((1 << shift) - 1)) << (8 - shift);
		return ((cH + (cH >> shift)) << 8) + cL + (cL >> shift);
	}
	return cc;
}

static void KeepSmallest(const Config& cfg, Levels& L, uint32_t* keys, int n, int weight, int shift, bool reverse, int maxSize)
{
	(void)cfg;
	if (n == 0)
		return;
	const int keep = n < maxSize ? n : maxSize;
	std::partial_sort(keys, keys + keep, keys + n);
	L.minErr = int(keys[0] >> 16) * weight;
	L.count = keep;
	for (int i = 0; i < keep; i++)
	{
		L.e[i].err = int(keys[i] >> 16) * weight;
		L.e[i].color = DecodeColor(keys[i] & 0xFFFFu, shift, reverse);
	}
}

/* src/SnippetLevelsBuffer.h:43-270 (candidate set as enumerated by the
   16-wide chunks of :433-530, the build the oracle is pinned to). */
void ChannelLevels(const Config& cfg, Levels& L, const Area& area, int offset, int weight, int water,
	int bits, int pbits, bool transparent, const uint8_t* table, bool single, int maxSize)
{
	const int shift = bits + int(pbits >= 0);
	const int rowSize = 1 << (2 * shift);

	uint32_t count;
	if (transparent)
	{
		count = area.active;
		if (!count)
		{
			L.minErr = 0;
			L.count = 1;
			L.e[0].err = 0;
			L.e[0].color = (pbits < 0) ? 0 : (pbits << (7 - bits));
			return;
		}
	}
	else
	{
		count = area.count;
	}

	const uint8_t* values[16];
	for (uint32_t i = 0; i < count; i++)
		values[i] = table + size_t(area.px[i][offset]) * rowSize;

	int32_t top = (water + weight - 1) / weight;
	if (!top)
		return;

	const int32_t d = WindowRadius(cfg, top);

	const int32_t L0 = int16_t(area.minmax[2 * offset + 0]);
	const int32_t H0 = int16_t(area.minmax[2 * offset + 1]);
	const bool reverse = (L0 != int16_t(area.bounds[2 * offset + 0]));

	if ((pbits < 0) || ((pbits >> 8) == (pbits & 1)))
	{
		if (L0 == H0)
		{
			if ((((L0 >> shift) ^ L0) & ((1 << (8 - shift)) - 1)) == 0)
			{
				if ((pbits < 0) || (((L0 >> (8 - shift)) & 1) == (pbits & 1)))
				{
					L.minErr = 0;
					L.count = 1;
					L.e[0].err = 0;
					L.e[0].color = (H0 << 8) + L0;
					return;
				}
			}
		}
	}

	Window win = MakeWindow(L0, H0, d, bits, shift);

	if (top > 0xFFFF)
		top = 0xFFFF;
	const uint32_t top16 = uint32_t(top) & 0xFFFF;

	PORT_COUNT(kScanCalls, 1);
	uint64_t scanned = 0;   /* window cells scored (work counters only) */
	auto sumAt = [&](int32_t c) -> uint32_t {
		scanned++;
		uint32_t s = 0;
		for (uint32_t i = 0; i < count; i++)
		{
			const uint32_t v = values[i][c];
			s += v * v;
		}
		return s > 0xFFFF ? 0xFFFF : s;
	};

	if (single)
	{
		/* :148-188 and :433-490 */
		uint32_t bestKey = 0xFFFFFFFFu;
		uint32_t bestSum = top16;
		for (int32_t iH = win.HL; iH < win.HH; iH++)
		{
			const int32_t cH = iH << shift;
			const int32_t hL = std::min(win.LH, iH) + cH;
			int32_t c = cH;
			do
			{
				const uint32_t tail = uint32_t(std::max(int32_t(0), Wsub(c | 15, hL | 7)));
				const uint32_t mask = Shr32(~0u, tail << 1);
				for (int j = 0; j < 16; j++)
				{
					if (!((mask >> (2 * j)) & 1))
						continue;
					const uint32_t s = sumAt(c + j);
					if (s < bestSum)
					{
						bestSum = s;
						bestKey = (s << 16) | uint32_t(c + j);
					}
				}
				c += 16;
			} while (c <= hL);
		}
		if (bestKey != 0xFFFFFFFFu)
		{
			const int e = int(bestKey >> 16) * weight;
			L.minErr = e;
			L.count = 1;
			L.e[0].err = e;
			L.e[0].color = DecodeColor(bestKey & 0xFFFFu, shift, reverse);
		}
		PORT_COUNT(kScanTerms, scanned * count);
		return;
	}

	static thread_local uint32_t keys[1 << 16];
	int n = 0;

	if (pbits < 0)
	{
		for (int32_t iH = win.HL; iH < win.HH; iH++)
		{
			const int32_t cH = iH << shift;
			const int32_t hL = win.LH + cH;
			int32_t c = cH;
			do
			{
				const uint32_t tail = Shr32(~0u, uint32_t(std::max(int32_t(0), Wsub(c | 15, hL | 7))) << 1);
				for (int j = 0; j < 16; j++)
				{
					if (!((tail >> (2 * j)) & 1))
						continue;
					const uint32_t s = sumAt(c + j);
					if (s < top16)
						keys[n++] = (s << 16) | uint32_t(c + j);
				}
				c += 16;
			} while (c <= hL);
		}
	}
	else
	{
		/* p-bit variants, :206-219 and :532-584 */
		const int pH = reverse ? (pbits & 1) : (pbits >> 8);
		const int pL = reverse ? (pbits >> 8) : (pbits & 1);
		for (int32_t iH = win.HL + pH; iH < win.HH; iH += 2)
		{
			const int32_t cH = iH << shift;
			const int32_t hL = win.LH + cH;
			int32_t c = cH;
			do
			{
				const uint32_t flags = Shr32(~0u, uint32_t(std::max(int32_t(0), Wsub(c | 31, hL | 7))));
				for (int j = 0; j < 16; j++)
				{
					if (!((flags >> (2 * j)) & 1))
						continue;
					const int32_t cc = c + pL + 2 * j;
					const uint32_t s = sumAt(cc);
					if (s < top16)
						keys[n++] = (s << 16) | uint32_t(cc);
				}
				c += 32;
			} while (c <= hL);
		}
	}

	PORT_COUNT(kScanTerms, scanned * count);
	(void)scanned;
	KeepSmallest(cfg, L, keys, n, weight, shift, reverse, maxSize);
}

/* src/SnippetLevelsBufferHalf.h:43-223 (nibble tables; the early stop after
   maxSize zero-error candidates keeps the first ones in ascending order,
   which equals the smallest keys of the full enumeration). */
void ChannelLevelsHalf(const Config& cfg, Levels& L, const Area& area, int offset, int weight, int water,
	int bits, int pbits, bool transparent, const uint8_t* table, int maxSize)
{
	const int shift = bits + 1;
	const int rowSize = 1 << (2 * shift - 1);

	uint32_t count;
	if (transparent)
	{
		count = area.active;
		if (!count)
		{
			L.minErr = 0;
			L.count = 1;
			L.e[0].err = 0;
			L.e[0].color = pbits << (7 - bits);
			return;
		}
	}
	else
	{
		count = area.count;
	}

	const uint8_t* values[16];
	for (uint32_t i = 0; i < count; i++)
		values[i] = table + size_t(area.px[i][offset]) * rowSize;

	int32_t top = (water + weight - 1) / weight;
	if (!top)
		return;

	const int32_t d = WindowRadius(cfg, top);

	const int32_t L0 = int16_t(area.minmax[2 * offset + 0]);
	const int32_t H0 = int16_t(area.minmax[2 * offset + 1]);
	const bool reverse = (L0 != int16_t(area.bounds[2 * offset + 0]));

	if ((pbits >> 8) == (pbits & 1))
	{
		if (L0 == H0)
		{
			if ((((L0 >> shift) ^ L0) & ((1 << (8 - shift)) - 1)) == 0)
			{
				if (((L0 >> (8 - shift)) & 1) == (pbits & 1))
				{
					L.minErr = 0;
					L.count = 1;
					L.e[0].err = 0;
					L.e[0].color = (H0 << 8) + L0;
					return;
				}
			}
		}
	}

	Window win = MakeWindow(L0, H0, d, bits, shift);

	top = std::min(top, int32_t(15 * 15 * 16 + 1));
	const int32_t top16 = int16_t(uint16_t(top));

	static thread_local uint32_t keys[1 << 16];
	int n = 0;

	const int pH = reverse ? (pbits & 1) : (pbits >> 8);
	const int pL = reverse ? (pbits >> 8) : (pbits & 1);

	PORT_COUNT(kScanCalls, 1);
	uint64_t scanned = 0;   /* window cells scored (work counters only) */
	for (int32_t iH = win.HL + pH; iH < win.HH; iH += 2)
	{
		const int32_t cH = iH << shift;
		const int32_t hL = win.LH + cH;
		int32_t c = cH;
		for (;;)
		{
			const uint32_t flags = Shr32(~0u, uint32_t(std::max(int32_t(0), Wsub(c | 31, hL | 7))));
			for (int j = 0; j < 16; j++)
			{
				if (!((flags >> (2 * j)) & 1))
					continue;
				const int32_t cc = c + pL + 2 * j;
				scanned++;
				int32_t s = 0;
				for (uint32_t i = 0; i < count; i++)
				{
					const int32_t v = (values[i][cc >> 1] >> ((cc & 1) << 2)) & 0xF;
					s += v * v;
				}
				if (top16 > s)
					keys[n++] = (uint32_t(s) << 16) | uint32_t(cc);
			}
			c += 32;
			if (c <= hL)
				continue;
			break;
		}
	}

	PORT_COUNT(kScanTerms, scanned * count);
	(void)scanned;
	KeepSmallest(cfg, L, keys, n, weight, shift, reverse, maxSize);
}

/* src/SnippetLevelsMinimum.h:117-311 */
int EstimateChannelLevels(const Config& cfg, const Area& area, int offset, int weight, int water,
	int bits, bool transparent, const uint8_t* table, const uint16_t* tower)
{
	const int shift = bits;
	const int rowSize = 1 << (2 * bits);
	const int towerSize = 1 << bits;

	uint32_t count;
	if (transparent)
	{
		count = area.active;
		if (!count)
			return 0;
	}
	else
	{
		count = area.count;
	}

	const uint8_t* values[16];
	const uint16_t* cuts[16];
	for (uint32_t i = 0; i < count; i++)
	{
		values[i] = table + size_t(area.px[i][offset]) * rowSize;
		cuts[i] = tower + size_t(area.px[i][offset]) * towerSize;
	}

	int32_t top = (water + weight - 1) / weight;
	if (!top)
		return 0;

	const int32_t d = WindowRadius(cfg, top);

	const int32_t L0 = int16_t(area.minmax[2 * offset + 0]);
	const int32_t H0 = int16_t(area.minmax[2 * offset + 1]);

	if (L0 == H0)
		return 0;
	if (bits == 7 && H0 - L0 <= 5)
		return 0;
	if (bits == 8 && H0 - L0 <= 3)
		return 0;

	Window win = MakeWindow(L0, H0, d, bits, shift);

	if (top > 0xFFFF)
		top = 0xFFFF;

	/* rows[iH]: saturating sum of the cut (row-minimum squared) values,
	   a lower bound for every candidate of row iH (:233-251). */
	PORT_COUNT(kEstCalls, 1);
	uint64_t terms = 0;   /* (cell or row, pixel) terms (work counters only) */
	uint32_t rows[256];
	for (int32_t iH = win.HL & ~15; iH < win.HH; iH++)
	{
		if (iH < 0)
			continue;
		terms += count;
		uint32_t s = 0;
		for (uint32_t i = 0; i < count; i++)
			s += cuts[i][iH];
		rows[iH] = s > 0xFFFF ? 0xFFFF : s;
	}

	int32_t best = top;
	for (int32_t iH = win.HL; iH < win.HH; iH++)
	{
		if (int32_t(rows[iH]) >= best)
			continue;
		const int32_t cH = iH << shift;
		uint32_t rowBest = 0xFFFF;
		for (int32_t iL = cH, hL = std::min(win.LH, iH) + cH; iL <= hL; iL += 32)
		{
			terms += 32 * count;
			for (int j = 0; j < 32; j++)
			{
				uint32_t s = 0;
				for (uint32_t i = 0; i < count; i++)
				{
					const uint32_t v = values[i][iL + j];
					s += v * v;
				}
				s = s > 0xFFFF ? 0xFFFF : s;
				rowBest = s < rowBest ? s : rowBest;
			}
		}
		best = std::min(best, int32_t(rowBest));
	}
	PORT_COUNT(kEstTerms, terms);
	(void)terms;
	return best * weight;
}

/* src/Bc7Core.cpp:564-619: stable sort by the 32-bit error. */
void RadixSortPartitions(Node* order, int n)
{
	std::stable_sort(order, order + n, [](const Node& a, const Node& b) { return uint32_t(a.err) < uint32_t(b.err); });
}

/* src/SnippetInsertRemoveZeroBit.h:5-17 */
uint64_t InsertZeroBit(uint64_t value, int index)
{
	uint64_t high = (~uint64_t(0) << index) & value;
	return (value ^ high) + (high << 1);
}

uint64_t RemoveZeroBit(uint64_t value, int index)
{
	uint64_t high = (~uint64_t(0) << index) & value;
	return (value ^ high) + (high >> 1);
}

static inline void SwapEndpoints(V8& mc)
{
	for (int c = 0; c < 4; c++)
	{
		int16_t t = mc.l[2 * c];
		mc.l[2 * c] = mc.l[2 * c + 1];
		mc.l[2 * c + 1] = t;
	}
}

/* src/Bc7Core.cpp:511-562 */
void AreaReduceTable2(const Area& area, V8& mc, uint64_t& indices)
{
	const int zerobit = area.zero * 2 + 1;
	if (indices & (uint64_t(1) << zerobit))
	{
		uint64_t mask = 0;
		for (uint32_t i = 0; i < area.count; i++)
			mask |= uint64_t(3) << (area.idx[i] << 1);
		indices ^= mask;
		SwapEndpoints(mc);
	}
}

void AreaReduceTable3(const Area& area, V8& mc, uint64_t& indices)
{
	const int zerobit = area.zero * 3 + 2;
	if (indices & (uint64_t(1) << zerobit))
	{
		uint64_t mask = 0;
		for (uint32_t i = 0; i < area.count; i++)
			mask |= uint64_t(7) << (area.idx[i] * 3);
		indices ^= mask;
		SwapEndpoints(mc);
	}
}

void AreaReduceTable4(V8& mc, uint64_t& indices)
{
	if (indices & (uint64_t(1) << 3))
	{
		indices = ~indices;
		SwapEndpoints(mc);
	}
}

/* ---------------------------------------------------------------------- */
/* Metrics, src/Metrics.cpp                                               */
/* ---------------------------------------------------------------------- */

void CompareBlocks(const Config& cfg, const Cell& a, const Cell& b, int& alpha, int& total)
{
	/* src/Metrics.cpp:7-111: masked, quantised, squared, weighted */
	int32_t sum[4] = { 0, 0, 0, 0 };
	for (int i = 0; i < 16; i++)
		for (int c = 0; c < 4; c++)
		{
			int q = cfg.Q(int(a.img[i][c]) - int(b.img[i][c]));
			q &= uint16_t(int16_t(int8_t(a.msk[i][c])));
			sum[c] += q * q;
		}
	const int w[4] = { cfg.wA, cfg.wG, cfg.wR, cfg.wB };
	int32_t t = 0;
	for (int c = 0; c < 4; c++)
	{
		sum[c] = Wmul(sum[c], w[c]);
		t = Wadd(t, sum[c]);
	}
	alpha = sum[0];
	total = t;
}

void CompareBlocksSSIM(const Config& cfg, const Cell& a, const Cell& b, double& alpha, double& color)
{
	/* src/Metrics.cpp:113-151 */
	int32_t sa[4] = { 0, 0, 0, 0 }, sb[4] = { 0, 0, 0, 0 }, sab[4] = { 0, 0, 0, 0 }, saa_sbb[4] = { 0, 0, 0, 0 };
	for (int i = 0; i < 16; i++)
		for (int c = 0; c < 4; c++)
		{
			const int32_t m = a.msk[i][c];
			const int32_t t = b.img[i][c] & m;
			const int32_t s = a.img[i][c] & m;
			sa[c] += t;
			sb[c] += s;
			sab[c] += t * s;
			saa_sbb[c] += t * t + s * s;
		}
	const double k1 = (0.01 * 255 * 16) * (0.01 * 255 * 16);
	const double k2 = k1 * 9;
	double r[4];
	for (int c = 0; c < 4; c++)
	{
		int32_t vab = int32_t(uint32_t(sab[c]) << 5);
		int32_t vaa = int32_t(uint32_t(saa_sbb[c]) << 4);
		int32_t sasb = Wmul(sa[c], sb[c]);
		sasb = Wadd(sasb, sasb);
		int32_t sasa_sbsb = Wadd(Wmul(sa[c], sa[c]), Wmul(sb[c], sb[c]));
		vab = Wsub(vab, sasb);
		vaa = Wsub(vaa, sasa_sbsb);
		r[c] = ((double(sasb) + k1) * (double(vab) + k2)) / ((double(sasa_sbsb) + k1) * (double(vaa) + k2));
	}
	const double ssim = r[1] * cfg.wG + r[2] * cfg.wR + r[3] * cfg.wB;
	alpha = r[0];
	color = ssim / cfg.wColor;
}

} // namespace nebc7_oracle
