/*
 * CPU oracle for the BC7 block encoder -- the nine mode encoders (test
 * infrastructure only; see port_tables.h).  Scalar restatement of reference
 * src/Bc7CoreMode{0,1,2,3,4,5,6,6Index2,7}.cpp: CompressBlockFast (bounding
 * box endpoints over every partition / rotation), CompressBlock (refinement
 * of the current winner over sorted per-channel candidate lists),
 * CompressBlockFull (estimate, order and search all partitions) and
 * FinalPackBlock (index selection and BPTC packing).  The nested candidate
 * loops keep the reference's visiting order, pruning tests and memoised
 * pair errors.
 */
#include "port_core.h"
#include "port_counters.h"

#include <string.h>

namespace nebc7_oracle {

namespace {

struct BitWriter
{
	uint64_t lo = 0, hi = 0;
	int pos = 0;

	void Put(uint64_t v, int n)
	{
		v &= (n == 64) ? ~uint64_t(0) : ((uint64_t(1) << n) - 1);
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

	void Store(uint8_t out[16]) const
	{
		memcpy(out, &lo, 8);
		memcpy(out + 8, &hi, 8);
	}
};

/* Writes per-pixel indices (bits each, pixel 0 first), dropping the zero
   MSB of the anchor pixels. */
void PutIndices(BitWriter& bw, uint64_t indices, int bits, const int* anchors, int nanchors)
{
	for (int i = 0; i < 16; i++)
	{
		bool anchor = false;
		for (int a = 0; a < nanchors; a++)
			anchor |= anchors[a] == i;
		const uint64_t v = (indices >> (i * bits)) & ((uint64_t(1) << bits) - 1);
		bw.Put(v, anchor ? bits - 1 : bits);
	}
}

inline void SetCh(uint8_t ep[8], int c, int color)
{
	ep[2 * c] = uint8_t(color & 0xFF);
	ep[2 * c + 1] = uint8_t((color >> 8) & 0xFF);
}

inline V8 Widen(const uint8_t ep[8])
{
	V8 v;
	for (int i = 0; i < 8; i++)
		v.l[i] = ep[i];
	return v;
}

inline void Pack(const V8& mc, uint8_t ep[8])
{
	PackEndpoints(mc, ep);
}

struct W4
{
	int w[4];
};

inline W4 Wt(const Config& c, bool a, bool g, bool r, bool b)
{
	W4 x;
	x.w[0] = a ? c.wA : 0;
	x.w[1] = g ? c.wG : 0;
	x.w[2] = r ? c.wR : 0;
	x.w[3] = b ? c.wB : 0;
	return x;
}

/* (count - active) * wA * D(0, alpha)^2 with the 2-bit table
   (src/Bc7CoreMode7.cpp:128, src/Bc7CoreMode6Index2.cpp:49) */
int TransparentError2(const Config& cfg, const Area& area, int alpha)
{
	int error = int(area.count - area.active);
	if (error)
	{
		error *= cfg.wA;
		const int v = cfg.lt->d2v8[alpha & 0xFFFF];
		error *= v * v;
	}
	return error;
}

/* same with the clamped 4-bit nibble table (src/Bc7CoreMode6.cpp:117) */
int TransparentError4(const Config& cfg, const Area& area, int alpha)
{
	int error = int(area.count - area.active);
	if (error)
	{
		error *= cfg.wA;
		const int v = (cfg.lt->d4h[(alpha & 0xFFFF) >> 1] >> ((alpha & 1) << 2)) & 0xF;
		error *= v * v;
	}
	return error;
}

inline int PackedAlpha(const uint8_t ep[8])
{
	return ep[0] | (ep[1] << 8);
}

/* The channel in the alpha-index slot for a mode 4/5 rotation
   (src/Bc7CoreMode4.cpp:21-48): 0 -> A, 1 -> R, 2 -> G, 3 -> B. */
inline int RotChannel(int rotation)
{
	static const int ch[4] = { 0, 2, 1, 3 };
	return ch[rotation & 3];
}

/* Storage (block) order <-> image order for rotated endpoints: swaps
   channel 0 with the rotated channel. */
inline void SwapRot(const uint8_t in[8], uint8_t out[8], int rotation)
{
	memcpy(out, in, 8);
	const int a = RotChannel(rotation);
	if (a)
	{
		out[0] = in[2 * a];
		out[1] = in[2 * a + 1];
		out[2 * a] = in[0];
		out[2 * a + 1] = in[1];
	}
}

/* Mode 4/5 error with separate color and alpha-slot indices
   (src/Bc7CoreMode4.cpp:159-492 / :494-839, src/Bc7CoreMode5.cpp:143-401).
   epImg: endpoints in image order; w: per-channel weights in image order;
   npix: pixels visited (Active for mode 4, 16 for mode 5); tail: add the
   (16 - Active) transparent-alpha term of mode 4. */
int RotError(const Config& cfg, const Area& area, const uint8_t epImg[8], int rotation, int colorBits, int alphaBits,
	const int w[4], int water, bool mode4)
{
	const int a = RotChannel(rotation);
	uint16_t vc[16][4], va[16][4];
	InterpolateLevels(epImg, colorBits, vc);
	InterpolateLevels(epImg, alphaBits, va);
	const int nc = 1 << colorBits, na = 1 << alphaBits;

	int sum = 0;
	const uint32_t npix = mode4 ? area.active : 16;
	uint32_t i = 0;
	for (; i < npix; i++)
	{
		int bestc = 0x7FFFFFFF;
		for (int k = 0; k < nc; k++)
		{
			int e = 0;
			for (int c = 0; c < 4; c++)
			{
				if (c == a)
					continue;
				const int q = cfg.Q(int(area.px[i][c]) - int(vc[k][c]));
				e += w[c] * ((q * q) & area.mk[i][c]);
			}
			bestc = e < bestc ? e : bestc;
		}
		int besta = 0x7FFFFFFF;
		for (int k = 0; k < na; k++)
		{
			const int q = cfg.Q(int(area.px[i][a]) - int(va[k][a]));
			const int e = w[a] * ((q * q) & area.mk[i][a]);
			besta = e < besta ? e : besta;
		}
		sum += besta;
		sum += bestc;
		if (!(water > sum))
		{
			PORT_COUNT(kErrCalls, 1);
			PORT_COUNT(kErrTerms, uint64_t(i + 1) * (nc * 3 + na));
			return sum;
		}
	}
	PORT_COUNT(kErrCalls, 1);
	PORT_COUNT(kErrTerms, uint64_t(i) * (nc * 3 + na));
	if (mode4 && i < 16)
	{
		int m = epImg[0] < epImg[1] ? epImg[0] : epImg[1];
		const int q = cfg.Q(m);
		sum += q * q * (w[0] * int(16 - i));
	}
	return sum;
}

/* ---------------------------------------------------------------------- */
/* Modes 0-3: three opaque channels G, R, B with a shared index          */
/* ---------------------------------------------------------------------- */

struct Est3
{
	int ch1, ch2, ch3;
};

struct Opaque3Spec
{
	int bits;          /* LevelsBuffer bits */
	int indexBits;     /* 3 for modes 0/1, 2 for modes 2/3 */
	const uint8_t* table;
	int estBits;
	const uint8_t* estTable;
	const uint16_t* estTower;
};

struct Subset3
{
	Levels ch1, ch2, ch3;

	bool InitLevels(const Config& cfg, const Opaque3Spec& s, int pbits, const Area& area, int water, const Est3& est)
	{
		LevelsInit(ch1, cfg);
		LevelsInit(ch2, cfg);
		LevelsInit(ch3, cfg);
		ChannelLevels(cfg, ch1, area, 1, cfg.wG, water - est.ch2 - est.ch3, s.bits, pbits, false, s.table, false, 32);
		const int min1 = ch1.minErr;
		if (min1 >= water)
			return false;
		ChannelLevels(cfg, ch2, area, 2, cfg.wR, water - min1 - est.ch3, s.bits, pbits, false, s.table, false, 32);
		const int min2 = ch2.minErr;
		if (min1 + min2 >= water)
			return false;
		ChannelLevels(cfg, ch3, area, 3, cfg.wB, water - min1 - min2, s.bits, pbits, false, s.table, false, 32);
		const int min3 = ch3.minErr;
		if (min1 + min2 + min3 >= water)
			return false;
		return true;
	}

	/* src/Bc7CoreMode0.cpp:270-363 (identical in modes 1, 2, 3) */
	int TryVariants(const Config& cfg, const Opaque3Spec& s, const Area& area, V8& best, int water)
	{
		const int min1 = ch1.minErr, min2 = ch2.minErr, min3 = ch3.minErr;
		if (min1 + min2 + min3 >= water)
			return water;
		const int n1 = ch1.count, n2 = ch2.count, n3 = ch3.count;
		const W4 wGR = Wt(cfg, false, true, true, false);
		const W4 wGB = Wt(cfg, false, true, false, true);
		const W4 wGRB = Wt(cfg, false, true, true, true);
		int memGB[32];
		for (int i1 = 0; i1 < n1; i1++)
		{
			const int e1 = ch1.e[i1].err;
			if (e1 + min2 + min3 >= water)
				break;
			const int c1 = ch1.e[i1].color;
			for (int i = 0; i < n3; i++)
				memGB[i] = -1;
			for (int i2 = 0; i2 < n2; i2++)
			{
				int e2 = ch2.e[i2].err + e1;
				if (e2 + min3 >= water)
					break;
				const int c2 = ch2.e[i2].color;
				{
					uint8_t ep[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
					SetCh(ep, 1, c1);
					SetCh(ep, 2, c2);
					e2 = SubsetError(cfg, area, ep, s.indexBits, wGR.w, water - min3);
					if (e2 + min3 >= water)
						continue;
				}
				for (int i3 = 0; i3 < n3; i3++)
				{
					const int e3 = ch3.e[i3].err + e2;
					if (e3 >= water)
						break;
					const int c3 = ch3.e[i3].color;
					int egb = memGB[i3];
					if (egb < 0)
					{
						uint8_t ep[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
						SetCh(ep, 1, c1);
						SetCh(ep, 3, c3);
						egb = SubsetError(cfg, area, ep, s.indexBits, wGB.w, water - min2);
						memGB[i3] = egb;
					}
					if (egb + min2 >= water)
						continue;
					uint8_t ep[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
					SetCh(ep, 1, c1);
					SetCh(ep, 2, c2);
					SetCh(ep, 3, c3);
					const int err = SubsetError(cfg, area, ep, s.indexBits, wGRB.w, water);
					if (water > err)
					{
						water = err;
						best = Widen(ep);
					}
				}
			}
		}
		return water;
	}
};

/* A set of p-bit variants tried in order (src/Bc7CoreMode0.cpp:366-415):
   each variant's lists are built with the same starting water. */
struct Subsets3
{
	Subset3 sub[4];
	bool valid[4];
	int n;
	const int* pbits;

	bool InitLevels(const Config& cfg, const Opaque3Spec& s, const int* variants, int nvariants, const Area& area, int water, const Est3& est)
	{
		n = nvariants;
		pbits = variants;
		bool any = false;
		for (int v = 0; v < n; v++)
		{
			valid[v] = sub[v].InitLevels(cfg, s, pbits[v], area, water, est);
			any |= valid[v];
		}
		return any;
	}

	int TryVariants(const Config& cfg, const Opaque3Spec& s, const Area& area, V8& best, int water)
	{
		for (int v = 0; v < n; v++)
			if (valid[v])
				water = sub[v].TryVariants(cfg, s, area, best, water);
		return water;
	}
};

const int kPbits4[4] = { 0x0101, 0, 1, 1 << 8 };
const int kPbits2[2] = { 0x0101, 0 };
const int kPbitsNone[1] = { -1 };

int EstimateLevels3(const Config& cfg, const Opaque3Spec& s, const Area& area, int water, Est3& est)
{
	/* src/Bc7CoreMode0.cpp:500-530 */
	int error = 0;
	if (error < water)
	{
		const int l1 = EstimateChannelLevels(cfg, area, 1, cfg.wG, water - error, s.estBits, false, s.estTable, s.estTower);
		est.ch1 = l1;
		error += l1;
		if (error < water)
		{
			const int l2 = EstimateChannelLevels(cfg, area, 2, cfg.wR, water - error, s.estBits, false, s.estTable, s.estTower);
			est.ch2 = l2;
			error += l2;
			if (error < water)
			{
				const int l3 = EstimateChannelLevels(cfg, area, 3, cfg.wB, water - error, s.estBits, false, s.estTable, s.estTower);
				est.ch3 = l3;
				error += l3;
				if (error < water)
					return error;
			}
		}
	}
	return water;
}

/* Refinement of the current winner of a 2- or 3-subset opaque mode
   (src/Bc7CoreMode0.cpp:417-498 and the same in modes 1-3). */
void RefineOpaque(const Config& cfg, const Opaque3Spec& s, const int* variants, int nvariants, Cell& input, int nsubsets)
{
	const int p = int(input.bestParam);
	V8 mc[3] = { input.best0, input.best1, input.best2 };
	const Est3 est = { 0, 0, 0 };
	const W4 wGRB = Wt(cfg, false, true, true, true);
	const Selection& sel = *cfg.sel;

	int error = input.opaqueAlphaError;
	if (error < input.errTotal)
	{
		for (int si = 0; si < nsubsets; si++)
		{
			Area* area;
			if (nsubsets == 3)
				area = si == 0 ? &GetArea(cfg, input.a13[p], input.lazy13[p], input, sel.sel13[p])
					: si == 1 ? &GetArea(cfg, input.a23[p], input.lazy23[p], input, sel.sel23[p])
					: &GetArea(cfg, input.a33[p], input.lazy33[p], input, sel.sel33[p]);
			else
				area = si == 0 ? &GetArea(cfg, input.a12[p], input.lazy12[p], input, sel.sel12[p])
					: &GetArea(cfg, input.a22[p], input.lazy22[p], input, sel.sel22[p]);
			uint8_t ep[8];
			Pack(mc[si], ep);
			const int water = SubsetError(cfg, *area, ep, s.indexBits, wGRB.w, cfg.MaxColorError());
			if (water)
			{
				Subsets3 subs;
				if (subs.InitLevels(cfg, s, variants, nvariants, *area, water, est))
					error += subs.TryVariants(cfg, s, *area, mc[si], water);
				else
					error += water;
			}
		}
		if (input.errTotal > error)
		{
			input.errTotal = error;
			input.best0 = mc[0];
			input.best1 = mc[1];
			if (nsubsets == 3)
				input.best2 = mc[2];
		}
	}
}

/* Mode 0 / 2 full search: estimate every partition, order, search
   (src/Bc7CoreMode0.cpp:532-642, src/Bc7CoreMode2.cpp:456-566). */
void FullThreeSubsets(const Config& cfg, const Opaque3Spec& s, const int* variants, int nvariants, Cell& input, int modeId, int npartitions)
{
	Node order[64];
	Est3 est1[64], est2[64], est3[64];
	int lines2[64], lines3[64];
	const int step = input.denoiseStep;
	const Selection& sel = *cfg.sel;

	int count = 0;
	for (int p = 0; p < npartitions; p++)
	{
		if (input.personalMode == uint32_t(modeId) && input.personalParam == uint64_t(p))
			continue;
		Area& area1 = GetArea(cfg, input.a13[p], input.lazy13[p], input, sel.sel13[p]);
		const int water1 = input.errTotal - step - input.opaqueAlphaError;
		const int line1 = EstimateLevels3(cfg, s, area1, water1, est1[p]);
		if (line1 < water1)
		{
			Area& area2 = GetArea(cfg, input.a23[p], input.lazy23[p], input, sel.sel23[p]);
			const int water2 = water1 - line1;
			const int line2 = EstimateLevels3(cfg, s, area2, water2, est2[p]);
			if (line2 < water2)
			{
				Area& area3 = GetArea(cfg, input.a33[p], input.lazy33[p], input, sel.sel33[p]);
				const int water3 = water2 - line2;
				const int line3 = EstimateLevels3(cfg, s, area3, water3, est3[p]);
				if (line3 < water3)
				{
					lines2[p] = line2;
					lines3[p] = line3;
					order[count].err = input.opaqueAlphaError + line1 + line2 + line3 + step;
					order[count].color = p;
					count++;
				}
			}
		}
	}

	RadixSortPartitions(order, count);

	for (int i = 0; i < count; i++)
	{
		if (order[i].err < input.errTotal)
		{
			const int p = order[i].color;
			V8 mc0 = V8Zero(), mc1 = V8Zero(), mc2 = V8Zero();
			const int line3 = lines3[p];
			Area& area1 = GetArea(cfg, input.a13[p], input.lazy13[p], input, sel.sel13[p]);
			const int water1 = input.errTotal - step - input.opaqueAlphaError - lines2[p] - line3;
			Subsets3 subs1;
			if (subs1.InitLevels(cfg, s, variants, nvariants, area1, water1, est1[p]))
			{
				int error = subs1.TryVariants(cfg, s, area1, mc0, water1);
				if (error < water1)
				{
					error += input.opaqueAlphaError;
					Area& area2 = GetArea(cfg, input.a23[p], input.lazy23[p], input, sel.sel23[p]);
					const int water2 = input.errTotal - step - error - line3;
					Subsets3 subs2;
					if (subs2.InitLevels(cfg, s, variants, nvariants, area2, water2, est2[p]))
					{
						error += subs2.TryVariants(cfg, s, area2, mc1, water2);
						if (error < input.errTotal - step - line3)
						{
							Area& area3 = GetArea(cfg, input.a33[p], input.lazy33[p], input, sel.sel33[p]);
							const int water3 = input.errTotal - step - error;
							Subsets3 subs3;
							if (subs3.InitLevels(cfg, s, variants, nvariants, area3, water3, est3[p]))
							{
								error += subs3.TryVariants(cfg, s, area3, mc2, water3);
								if (input.errTotal > error + step)
								{
									input.errTotal = error;
									input.best0 = mc0;
									input.best1 = mc1;
									input.best2 = mc2;
									input.bestParam = uint64_t(p);
									input.bestMode = uint32_t(modeId);
									if (error <= input.opaqueAlphaError)
										return;
								}
							}
						}
					}
				}
			}
		}
	}
}

/* Mode 1 / 3 full search (src/Bc7CoreMode1.cpp:473-571, src/Bc7CoreMode3.cpp:471-569). */
void FullTwoSubsets(const Config& cfg, const Opaque3Spec& s, const int* variants, int nvariants, Cell& input, int modeId)
{
	Node order[64];
	int lines1[64], lines2[64];
	const int step = input.denoiseStep;
	const Selection& sel = *cfg.sel;

	int count = 0;
	for (int p = 0; p < 64; p++)
	{
		if (input.personalMode == uint32_t(modeId) && input.personalParam == uint64_t(p))
			continue;
		GetArea(cfg, input.a12[p], input.lazy12[p], input, sel.sel12[p]);
		const int water1 = input.errTotal - step - input.opaqueAlphaError;
		/* AreaGetBestPca3 (src/Bc7Core.cpp:494): 0 without OPTION_PCA */
		const int line1 = cfg.pca ? PcaBound(cfg, input.a12[p], 3) : 0;
		if (line1 < water1)
		{
			GetArea(cfg, input.a22[p], input.lazy22[p], input, sel.sel22[p]);
			const int water2 = water1 - line1;
			const int line2 = cfg.pca ? PcaBound(cfg, input.a22[p], 3) : 0;
			if (line2 < water2)
			{
				lines1[p] = line1;
				lines2[p] = line2;
				order[count].err = input.opaqueAlphaError + line1 + line2 + step;
				order[count].color = p;
				count++;
			}
		}
	}

	RadixSortPartitions(order, count);

	for (int i = 0; i < count; i++)
	{
		if (order[i].err < input.errTotal)
		{
			const int p = order[i].color;
			V8 mc0 = V8Zero(), mc1 = V8Zero();
			Area& area1 = GetArea(cfg, input.a12[p], input.lazy12[p], input, sel.sel12[p]);
			Area& area2 = GetArea(cfg, input.a22[p], input.lazy22[p], input, sel.sel22[p]);
			int line1 = lines1[p];
			int line2 = lines2[p];
			Est3 e1, e2;
			int water1 = input.errTotal - step - input.opaqueAlphaError - line2;
			{
				const int l = EstimateLevels3(cfg, s, area1, water1, e1);
				line1 = line1 > l ? line1 : l;
			}
			if (line1 < water1)
			{
				int water2 = water1 - line1;
				{
					const int l = EstimateLevels3(cfg, s, area2, water2, e2);
					line2 = line2 > l ? line2 : l;
				}
				if (line2 < water2)
				{
					water1 = input.errTotal - step - input.opaqueAlphaError - line2;
					Subsets3 subs1;
					if (subs1.InitLevels(cfg, s, variants, nvariants, area1, water1, e1))
					{
						int error = subs1.TryVariants(cfg, s, area1, mc0, water1);
						if (error < water1)
						{
							error += input.opaqueAlphaError;
							water2 = input.errTotal - step - error;
							Subsets3 subs2;
							if (subs2.InitLevels(cfg, s, variants, nvariants, area2, water2, e2))
							{
								error += subs2.TryVariants(cfg, s, area2, mc1, water2);
								if (input.errTotal > error + step)
								{
									input.errTotal = error;
									input.best0 = mc0;
									input.best1 = mc1;
									input.bestParam = uint64_t(p);
									input.bestMode = uint32_t(modeId);
									if (error <= input.opaqueAlphaError)
										return;
								}
							}
						}
					}
				}
			}
		}
	}
}

/* FinalPack helpers for the opaque subset modes: ComputeOpaqueSubsetTable3
   (src/SnippetComputeOpaqueSubset3.h:637) and ComputeSubsetTable2<opaque>
   (src/SnippetComputeOpaqueSubset2.h:609). */
int OpaqueTable(const Config& cfg, const Area& area, V8 mc, int indexBits, uint64_t& indices, bool forceOpaque, int* errorAlphaOut)
{
	if (forceOpaque)
	{
		mc.l[0] |= 255;
		mc.l[1] |= 255;
	}
	uint8_t ep[8];
	Pack(mc, ep);
	uint16_t vals[16][4];
	InterpolateLevels(ep, indexBits, vals);
	const int w[4] = { cfg.wA, cfg.wG, cfg.wR, cfg.wB };
	int best[16];
	const int error = ComputeSubsetTable(cfg, area, w, 1 << indexBits, vals, best);
	for (uint32_t i = 0; i < area.count; i++)
		indices |= uint64_t(uint32_t(best[i])) << (area.idx[i] * indexBits);
	if (errorAlphaOut)
	{
		int errorAlpha = 0;
		for (uint32_t i = 0; i < area.count; i++)
		{
			int da = int(vals[best[i]][0]) - int(area.px[i][0]);
			da = da < 0 ? -da : da;
			if (!cfg.denoise)
				da = da > 0x7F ? 0x7F : da;
			else
				da >>= cfg.denoise;
			errorAlpha += da * da;
		}
		*errorAlphaOut = errorAlpha * cfg.wA;
	}
	return error;
}

} // namespace

/* ======================================================================= */
/* Mode 0: 3 subsets, 16 partitions, RGB 4 + unique p, 3-bit index         */
/* ======================================================================= */
namespace mode0 {

static Opaque3Spec Spec(const Config& cfg)
{
	return Opaque3Spec{ 4, 3, cfg.lt->d3v5, 5, cfg.lt->d3v5, cfg.lt->c3v5 };
}

void FinalPack(const Config& cfg, uint8_t* out, Cell& input)
{
	/* src/Bc7CoreMode0.cpp:92-167 */
	const Selection& sel = *cfg.sel;
	const int p = int(input.bestParam);
	Area& a1 = GetArea(cfg, input.a13[p], input.lazy13[p], input, sel.sel13[p]);
	Area& a2 = GetArea(cfg, input.a23[p], input.lazy23[p], input, sel.sel23[p]);
	Area& a3 = GetArea(cfg, input.a33[p], input.lazy33[p], input, sel.sel33[p]);
	V8 mc0 = input.best0, mc1 = input.best1, mc2 = input.best2;
	uint64_t indices = 0;
	input.errAlpha = input.opaqueAlphaError;
	input.errTotal = OpaqueTable(cfg, a1, mc0, 3, indices, true, nullptr);
	input.errTotal += OpaqueTable(cfg, a2, mc1, 3, indices, true, nullptr);
	input.errTotal += OpaqueTable(cfg, a3, mc2, 3, indices, true, nullptr);
	AreaReduceTable3(a1, mc0, indices);
	AreaReduceTable3(a2, mc1, indices);
	AreaReduceTable3(a3, mc2, indices);

	const V8* mc[3] = { &mc0, &mc1, &mc2 };
	BitWriter bw;
	bw.Put(1, 1);
	bw.Put(uint64_t(p), 4);
	const int ch[3] = { 2, 1, 3 };
	for (int c = 0; c < 3; c++)
		for (int s = 0; s < 3; s++)
			for (int k = 0; k < 2; k++)
				bw.Put(uint64_t((mc[s]->l[2 * ch[c] + k] >> 4) & 0xF), 4);
	for (int s = 0; s < 3; s++)
		for (int k = 0; k < 2; k++)
			bw.Put(uint64_t((mc[s]->l[2 + k] >> 3) & 1), 1);
	const int anchors[3] = { 0, kAnchor2of3[p], kAnchor3of3[p] };
	PutIndices(bw, indices, 3, anchors, 3);
	bw.Store(out);
}

static int SubsetFast(const Config& cfg, const Area& area, V8& mc, int water)
{
	/* src/Bc7CoreMode0.cpp:169-187 */
	V8 m;
	memcpy(m.l, area.bounds, sizeof(m.l));
	const int p0 = m.l[2] & 8, p1 = m.l[3] & 8;
	for (int i = 0; i < 8; i++)
	{
		int v = m.l[i] & 0xF0;
		v |= v >> 5;
		v |= (i & 1) ? p1 : p0;
		m.l[i] = int16_t(v);
	}
	mc = m;
	uint8_t ep[8];
	Pack(mc, ep);
	const W4 w = Wt(cfg, false, true, true, true);
	return SubsetError(cfg, area, ep, 3, w.w, water);
}

void Fast(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode0.cpp:189-235 */
	const int step = input.denoiseStep;
	const Selection& sel = *cfg.sel;
	for (int p = 0; p < 16; p++)
	{
		V8 mc0 = V8Zero(), mc1 = V8Zero(), mc2 = V8Zero();
		int error = input.opaqueAlphaError + step;
		if (error < input.errTotal)
		{
			Area& a1 = GetArea(cfg, input.a13[p], input.lazy13[p], input, sel.sel13[p]);
			error += SubsetFast(cfg, a1, mc0, input.errTotal - error);
			if (error < input.errTotal)
			{
				Area& a2 = GetArea(cfg, input.a23[p], input.lazy23[p], input, sel.sel23[p]);
				error += SubsetFast(cfg, a2, mc1, input.errTotal - error);
				if (error < input.errTotal)
				{
					Area& a3 = GetArea(cfg, input.a33[p], input.lazy33[p], input, sel.sel33[p]);
					error += SubsetFast(cfg, a3, mc2, input.errTotal - error);
					if (input.errTotal > error)
					{
						input.errTotal = error - step;
						input.best0 = mc0;
						input.best1 = mc1;
						input.best2 = mc2;
						input.bestParam = uint64_t(p);
						input.bestMode = 0;
						if (error <= input.opaqueAlphaError + step)
							return;
					}
				}
			}
		}
	}
}

void Refine(const Config& cfg, Cell& input)
{
	RefineOpaque(cfg, Spec(cfg), kPbits4, 4, input, 3);
}

void Full(const Config& cfg, Cell& input)
{
	FullThreeSubsets(cfg, Spec(cfg), kPbits4, 4, input, 0, 16);
}

} // namespace mode0

/* ======================================================================= */
/* Mode 1: 2 subsets, 64 partitions, RGB 6 + shared p, 3-bit index          */
/* ======================================================================= */
namespace mode1 {

static Opaque3Spec Spec(const Config& cfg)
{
	return Opaque3Spec{ 6, 3, cfg.lt->d3v7s, 7, cfg.lt->d3v7s, cfg.lt->c3v7s };
}

void FinalPack(const Config& cfg, uint8_t* out, Cell& input)
{
	/* src/Bc7CoreMode1.cpp:83-139 */
	const Selection& sel = *cfg.sel;
	const int p = int(input.bestParam);
	Area& a1 = GetArea(cfg, input.a12[p], input.lazy12[p], input, sel.sel12[p]);
	Area& a2 = GetArea(cfg, input.a22[p], input.lazy22[p], input, sel.sel22[p]);
	V8 mc0 = input.best0, mc1 = input.best1;
	uint64_t indices = 0;
	input.errAlpha = input.opaqueAlphaError;
	input.errTotal = OpaqueTable(cfg, a1, mc0, 3, indices, true, nullptr);
	input.errTotal += OpaqueTable(cfg, a2, mc1, 3, indices, true, nullptr);
	AreaReduceTable3(a1, mc0, indices);
	AreaReduceTable3(a2, mc1, indices);

	const V8* mc[2] = { &mc0, &mc1 };
	BitWriter bw;
	bw.Put(2, 2);
	bw.Put(uint64_t(p), 6);
	const int ch[3] = { 2, 1, 3 };
	for (int c = 0; c < 3; c++)
		for (int s = 0; s < 2; s++)
			for (int k = 0; k < 2; k++)
				bw.Put(uint64_t((mc[s]->l[2 * ch[c] + k] >> 2) & 0x3F), 6);
	for (int s = 0; s < 2; s++)
		bw.Put(uint64_t((mc[s]->l[2] >> 1) & 1), 1);
	const int anchors[2] = { 0, kAnchor2of2[p] };
	PutIndices(bw, indices, 3, anchors, 2);
	bw.Store(out);
}

static int SubsetFast(const Config& cfg, const Area& area, V8& mc, int water)
{
	/* src/Bc7CoreMode1.cpp:141-174 */
	V8 m;
	memcpy(m.l, area.bounds, sizeof(m.l));
	for (int i = 0; i < 8; i++)
	{
		int v = m.l[i] & 0xFC;
		v |= v >> 7;
		m.l[i] = int16_t(v);
	}
	mc = m;
	const W4 w = Wt(cfg, false, true, true, true);
	uint8_t ep[8];
	Pack(mc, ep);
	const int e0 = SubsetError(cfg, area, ep, 3, w.w, water);
	if (water > e0)
		water = e0;
	V8 mp = mc;
	for (int i = 0; i < 8; i++)
		mp.l[i] = int16_t(mp.l[i] | 2);
	Pack(mp, ep);
	const int e1 = SubsetError(cfg, area, ep, 3, w.w, water);
	if (water > e1)
	{
		water = e1;
		mc = mp;
	}
	return water;
}

void Fast(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode1.cpp:176-213 */
	const int step = input.denoiseStep;
	const Selection& sel = *cfg.sel;
	for (int p = 0; p < 64; p++)
	{
		V8 mc0 = V8Zero(), mc1 = V8Zero();
		int error = input.opaqueAlphaError + step;
		if (error < input.errTotal)
		{
			Area& a1 = GetArea(cfg, input.a12[p], input.lazy12[p], input, sel.sel12[p]);
			error += SubsetFast(cfg, a1, mc0, input.errTotal - error);
			if (error < input.errTotal)
			{
				Area& a2 = GetArea(cfg, input.a22[p], input.lazy22[p], input, sel.sel22[p]);
				error += SubsetFast(cfg, a2, mc1, input.errTotal - error);
				if (input.errTotal > error)
				{
					input.errTotal = error - step;
					input.best0 = mc0;
					input.best1 = mc1;
					input.bestParam = uint64_t(p);
					input.bestMode = 1;
					if (error <= input.opaqueAlphaError + step)
						return;
				}
			}
		}
	}
}

void Refine(const Config& cfg, Cell& input)
{
	RefineOpaque(cfg, Spec(cfg), kPbits2, 2, input, 2);
}

void Full(const Config& cfg, Cell& input)
{
	FullTwoSubsets(cfg, Spec(cfg), kPbits2, 2, input, 1);
}

} // namespace mode1

/* ======================================================================= */
/* Mode 2: 3 subsets, 64 partitions, RGB 5, 2-bit index                     */
/* ======================================================================= */
namespace mode2 {

static Opaque3Spec Spec(const Config& cfg)
{
	return Opaque3Spec{ 5, 2, cfg.lt->d2v5, 5, cfg.lt->d2v5, cfg.lt->c2v5 };
}

void FinalPack(const Config& cfg, uint8_t* out, Cell& input)
{
	/* src/Bc7CoreMode2.cpp:85-148 */
	const Selection& sel = *cfg.sel;
	const int p = int(input.bestParam);
	Area& a1 = GetArea(cfg, input.a13[p], input.lazy13[p], input, sel.sel13[p]);
	Area& a2 = GetArea(cfg, input.a23[p], input.lazy23[p], input, sel.sel23[p]);
	Area& a3 = GetArea(cfg, input.a33[p], input.lazy33[p], input, sel.sel33[p]);
	V8 mc0 = input.best0, mc1 = input.best1, mc2 = input.best2;
	uint64_t indices = 0;
	input.errAlpha = input.opaqueAlphaError;
	input.errTotal = OpaqueTable(cfg, a1, mc0, 2, indices, true, nullptr);
	input.errTotal += OpaqueTable(cfg, a2, mc1, 2, indices, true, nullptr);
	input.errTotal += OpaqueTable(cfg, a3, mc2, 2, indices, true, nullptr);
	AreaReduceTable2(a1, mc0, indices);
	AreaReduceTable2(a2, mc1, indices);
	AreaReduceTable2(a3, mc2, indices);

	const V8* mc[3] = { &mc0, &mc1, &mc2 };
	BitWriter bw;
	bw.Put(4, 3);
	bw.Put(uint64_t(p), 6);
	const int ch[3] = { 2, 1, 3 };
	for (int c = 0; c < 3; c++)
		for (int s = 0; s < 3; s++)
			for (int k = 0; k < 2; k++)
				bw.Put(uint64_t((mc[s]->l[2 * ch[c] + k] >> 3) & 0x1F), 5);
	const int anchors[3] = { 0, kAnchor2of3[p], kAnchor3of3[p] };
	PutIndices(bw, indices, 2, anchors, 3);
	bw.Store(out);
}

static int SubsetFast(const Config& cfg, const Area& area, V8& mc, int water)
{
	/* src/Bc7CoreMode2.cpp:150-163 */
	V8 m;
	memcpy(m.l, area.bounds, sizeof(m.l));
	for (int i = 0; i < 8; i++)
	{
		int v = m.l[i] & 0xF8;
		v |= v >> 5;
		m.l[i] = int16_t(v);
	}
	mc = m;
	const W4 w = Wt(cfg, false, true, true, true);
	uint8_t ep[8];
	Pack(mc, ep);
	return SubsetError(cfg, area, ep, 2, w.w, water);
}

void Fast(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode2.cpp:165-211 */
	const int step = input.denoiseStep;
	const Selection& sel = *cfg.sel;
	for (int p = 0; p < 64; p++)
	{
		V8 mc0 = V8Zero(), mc1 = V8Zero(), mc2 = V8Zero();
		int error = input.opaqueAlphaError + step;
		if (error < input.errTotal)
		{
			Area& a1 = GetArea(cfg, input.a13[p], input.lazy13[p], input, sel.sel13[p]);
			error += SubsetFast(cfg, a1, mc0, input.errTotal - error);
			if (error < input.errTotal)
			{
				Area& a2 = GetArea(cfg, input.a23[p], input.lazy23[p], input, sel.sel23[p]);
				error += SubsetFast(cfg, a2, mc1, input.errTotal - error);
				if (error < input.errTotal)
				{
					Area& a3 = GetArea(cfg, input.a33[p], input.lazy33[p], input, sel.sel33[p]);
					error += SubsetFast(cfg, a3, mc2, input.errTotal - error);
					if (input.errTotal > error)
					{
						input.errTotal = error - step;
						input.best0 = mc0;
						input.best1 = mc1;
						input.best2 = mc2;
						input.bestParam = uint64_t(p);
						input.bestMode = 2;
						if (error <= input.opaqueAlphaError + step)
							return;
					}
				}
			}
		}
	}
}

void Refine(const Config& cfg, Cell& input)
{
	RefineOpaque(cfg, Spec(cfg), kPbitsNone, 1, input, 3);
}

void Full(const Config& cfg, Cell& input)
{
	FullThreeSubsets(cfg, Spec(cfg), kPbitsNone, 1, input, 2, 64);
}

} // namespace mode2

/* ======================================================================= */
/* Mode 3: 2 subsets, 64 partitions, RGB 7 + unique p, 2-bit index          */
/* ======================================================================= */
namespace mode3 {

static Opaque3Spec Spec(const Config& cfg)
{
	return Opaque3Spec{ 7, 2, cfg.lt->d2v8, 8, cfg.lt->d2v8, cfg.lt->c2v8 };
}

void FinalPack(const Config& cfg, uint8_t* out, Cell& input)
{
	/* src/Bc7CoreMode3.cpp:83-138 */
	const Selection& sel = *cfg.sel;
	const int p = int(input.bestParam);
	Area& a1 = GetArea(cfg, input.a12[p], input.lazy12[p], input, sel.sel12[p]);
	Area& a2 = GetArea(cfg, input.a22[p], input.lazy22[p], input, sel.sel22[p]);
	V8 mc0 = input.best0, mc1 = input.best1;
	uint64_t indices = 0;
	input.errAlpha = input.opaqueAlphaError;
	input.errTotal = OpaqueTable(cfg, a1, mc0, 2, indices, true, nullptr);
	input.errTotal += OpaqueTable(cfg, a2, mc1, 2, indices, true, nullptr);
	AreaReduceTable2(a1, mc0, indices);
	AreaReduceTable2(a2, mc1, indices);

	const V8* mc[2] = { &mc0, &mc1 };
	BitWriter bw;
	bw.Put(8, 4);
	bw.Put(uint64_t(p), 6);
	const int ch[3] = { 2, 1, 3 };
	for (int c = 0; c < 3; c++)
		for (int s = 0; s < 2; s++)
			for (int k = 0; k < 2; k++)
				bw.Put(uint64_t((mc[s]->l[2 * ch[c] + k] >> 1) & 0x7F), 7);
	for (int s = 0; s < 2; s++)
		for (int k = 0; k < 2; k++)
			bw.Put(uint64_t(mc[s]->l[2 + k] & 1), 1);
	const int anchors[2] = { 0, kAnchor2of2[p] };
	PutIndices(bw, indices, 2, anchors, 2);
	bw.Store(out);
}

static int SubsetFast(const Config& cfg, const Area& area, V8& mc, int water)
{
	/* src/Bc7CoreMode3.cpp:140-156 */
	V8 m;
	memcpy(m.l, area.bounds, sizeof(m.l));
	const int p0 = m.l[2] & 1, p1 = m.l[3] & 1;
	for (int i = 0; i < 8; i++)
		m.l[i] = int16_t((m.l[i] & 0xFE) | ((i & 1) ? p1 : p0));
	mc = m;
	const W4 w = Wt(cfg, false, true, true, true);
	uint8_t ep[8];
	Pack(mc, ep);
	return SubsetError(cfg, area, ep, 2, w.w, water);
}

void Fast(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode3.cpp:158-195 */
	const int step = input.denoiseStep;
	const Selection& sel = *cfg.sel;
	for (int p = 0; p < 64; p++)
	{
		V8 mc0 = V8Zero(), mc1 = V8Zero();
		int error = input.opaqueAlphaError + step;
		if (error < input.errTotal)
		{
			Area& a1 = GetArea(cfg, input.a12[p], input.lazy12[p], input, sel.sel12[p]);
			error += SubsetFast(cfg, a1, mc0, input.errTotal - error);
			if (error < input.errTotal)
			{
				Area& a2 = GetArea(cfg, input.a22[p], input.lazy22[p], input, sel.sel22[p]);
				error += SubsetFast(cfg, a2, mc1, input.errTotal - error);
				if (input.errTotal > error)
				{
					input.errTotal = error - step;
					input.best0 = mc0;
					input.best1 = mc1;
					input.bestParam = uint64_t(p);
					input.bestMode = 3;
					if (error <= input.opaqueAlphaError + step)
						return;
				}
			}
		}
	}
}

void Refine(const Config& cfg, Cell& input)
{
	RefineOpaque(cfg, Spec(cfg), kPbits4, 4, input, 2);
}

void Full(const Config& cfg, Cell& input)
{
	FullTwoSubsets(cfg, Spec(cfg), kPbits4, 4, input, 3);
}

} // namespace mode3

/* ======================================================================= */
/* Modes 4 and 5: one subset, rotation, separate color / alpha indices      */
/* ======================================================================= */
namespace {

struct RotSpec
{
	bool mode4;
	int colorBits, alphaBits;   /* index bits of the color set and the alpha slot */
	int cbits, abits;           /* endpoint bits of colors and of the alpha slot */
	const uint8_t* colorTable;  /* LevelsBuffer table for color channels */
	const uint8_t* alphaTable;  /* single-best table for the alpha slot */
};

RotSpec SpecFor(const Config& cfg, bool mode4, int rotation)
{
	if (mode4)
	{
		if (rotation & 4)
			return RotSpec{ true, 3, 2, 5, 6, cfg.lt->d3v5, cfg.lt->d2v6 };
		return RotSpec{ true, 2, 3, 5, 6, cfg.lt->d2v5, cfg.lt->d3v6 };
	}
	return RotSpec{ false, 2, 2, 7, 8, cfg.lt->d2v7, cfg.lt->d2v8 };
}

struct RotSubset
{
	Levels ch[4];

	/* src/Bc7CoreMode4.cpp:1264-1322 / :1505-1563, src/Bc7CoreMode5.cpp:628-686 */
	bool InitLevels(const Config& cfg, const RotSpec& s, const Area& area, int water, int rotation)
	{
		for (int c = 0; c < 4; c++)
			LevelsInit(ch[c], cfg);
		const int a = RotChannel(rotation);
		const int wts[4] = { cfg.wA, cfg.wG, cfg.wR, cfg.wB };
		int used = 0;
		for (int c = 0; c < 4; c++)
		{
			if (c == 0 && area.opaque)
			{
				ch[0].minErr = 0;
				ch[0].count = 1;
				ch[0].e[0].err = 0;
				ch[0].e[0].color = 0xFFFF;
			}
			else
			{
				const bool transparent = c != 0;
				if (c == a)
					ChannelLevels(cfg, ch[c], area, c, wts[c], water - used, s.abits, -1, transparent, s.alphaTable, true, 32);
				else
					ChannelLevels(cfg, ch[c], area, c, wts[c], water - used, s.cbits, -1, transparent, s.colorTable, false, 32);
			}
			used += ch[c].minErr;
			if (used >= water)
				return false;
		}
		return true;
	}

	int Err(const Config& cfg, const RotSpec& s, const Area& area, const uint8_t ep[8], int rotation, const W4& w, int water) const
	{
		return RotError(cfg, area, ep, rotation, s.colorBits, s.alphaBits, w.w, water, s.mode4);
	}

	/* src/Bc7CoreMode4.cpp:1324-1495 / :1565-1736, src/Bc7CoreMode5.cpp:688-859 */
	int TryVariants(const Config& cfg, const RotSpec& s, const Area& area, uint8_t bestStorage[8], int water, int rot)
	{
		const int minA = ch[0].minErr, minG = ch[1].minErr, minR = ch[2].minErr, minB = ch[3].minErr;
		if (minA + minG + minR + minB >= water)
			return water;
		const int nA = (rot == 0) ? 1 : ch[0].count;
		const int nG = (rot == 2) ? 1 : ch[1].count;
		const int nR = (rot == 1) ? 1 : ch[2].count;
		const int nB = (rot == 3) ? 1 : ch[3].count;
		const W4 wAG = Wt(cfg, true, true, false, false);
		const W4 wAR = Wt(cfg, true, false, true, false);
		const W4 wAGR = Wt(cfg, true, true, true, false);
		const W4 wAGB = Wt(cfg, true, true, false, true);
		const W4 wAGRB = Wt(cfg, true, true, true, true);
		int memAR[32], memAGB[32];

		for (int iA = 0; iA < nA; iA++)
		{
			const int eA = ch[0].e[iA].err;
			if (eA + minG + minR + minB >= water)
				break;
			const int cA = ch[0].e[iA].color;
			for (int i = 0; i < nR; i++)
				memAR[i] = -1;
			for (int iG = 0; iG < nG; iG++)
			{
				int eG = ch[1].e[iG].err + eA;
				if (eG + minR + minB >= water)
					break;
				const int cG = ch[1].e[iG].color;
				if (rot == 1 || rot == 3)
				{
					uint8_t ep[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
					SetCh(ep, 0, cA);
					SetCh(ep, 1, cG);
					eG = Err(cfg, s, area, ep, rot, wAG, water - minR - minB);
					if (eG + minR + minB >= water)
						continue;
				}
				for (int i = 0; i < nB; i++)
					memAGB[i] = -1;
				for (int iR = 0; iR < nR; iR++)
				{
					int eR = ch[2].e[iR].err + eG;
					if (eR + minB >= water)
						break;
					const int cR = ch[2].e[iR].color;
					if (rot == 2 || rot == 3)
					{
						int ear = memAR[iR];
						if (ear < 0)
						{
							uint8_t ep[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
							SetCh(ep, 0, cA);
							SetCh(ep, 2, cR);
							ear = Err(cfg, s, area, ep, rot, wAR, water - minG - minB);
							memAR[iR] = ear;
						}
						if (ear + minG + minB >= water)
							continue;
						if (rot == 2)
							eR = ear + ch[1].e[iG].err;
					}
					if (rot == 0 || rot == 3)
					{
						uint8_t ep[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
						SetCh(ep, 0, cA);
						SetCh(ep, 1, cG);
						SetCh(ep, 2, cR);
						eR = Err(cfg, s, area, ep, rot, wAGR, water - minB);
						if (eR + minB >= water)
							continue;
					}
					for (int iB = 0; iB < nB; iB++)
					{
						int eB = ch[3].e[iB].err + eR;
						if (eB >= water)
							break;
						const int cB = ch[3].e[iB].color;
						if (rot != 3)
						{
							int eagb = memAGB[iB];
							if (eagb < 0)
							{
								uint8_t ep[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
								SetCh(ep, 0, cA);
								SetCh(ep, 1, cG);
								SetCh(ep, 3, cB);
								eagb = Err(cfg, s, area, ep, rot, wAGB, water - minR);
								memAGB[iB] = eagb;
							}
							if (eagb + minR >= water)
								continue;
							if (rot == 1)
								eB = eagb + ch[2].e[iR].err;
						}
						uint8_t ep[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
						SetCh(ep, 0, cA);
						SetCh(ep, 1, cG);
						SetCh(ep, 2, cR);
						SetCh(ep, 3, cB);
						if (rot == 0 || rot == 2)
							eB = Err(cfg, s, area, ep, rot, wAGRB, water);
						if (water > eB)
						{
							water = eB;
							SwapRot(ep, bestStorage, rot);
						}
					}
				}
			}
		}
		return water;
	}
};

int CompressRotSubset(const Config& cfg, bool mode4, const Area& area, uint8_t mcStorage[8], int water, int rotation)
{
	const RotSpec s = SpecFor(cfg, mode4, rotation);
	RotSubset sub;
	if (sub.InitLevels(cfg, s, area, water, rotation))
		water = sub.TryVariants(cfg, s, area, mcStorage, water, rotation & 3);
	return water;
}

/* FinalPack for modes 4 and 5 (src/Bc7CoreMode4.cpp:841-1193,
   src/Bc7CoreMode5.cpp:403-567). */
void FinalPackRot(const Config& cfg, uint8_t* out, Cell& input, bool mode4)
{
	const int rotation = int(input.bestParam);
	const RotSpec s = SpecFor(cfg, mode4, rotation);
	Area& area = input.area1;
	V8 mc = input.best0;
	uint8_t epS[8], epI[8];
	Pack(mc, epS);
	SwapRot(epS, epI, rotation);
	const int a = RotChannel(rotation);

	uint16_t vc[16][4], va[16][4];
	InterpolateLevels(epI, s.colorBits, vc);
	InterpolateLevels(epI, s.alphaBits, va);
	for (int k = 0; k < 16; k++)
	{
		vc[k][a] = 0;
		for (int c = 0; c < 4; c++)
			if (c != a)
				va[k][c] = 0;
	}
	int wc[4] = { cfg.wA, cfg.wG, cfg.wR, cfg.wB };
	int wa[4] = { 0, 0, 0, 0 };
	wa[a] = wc[a];
	wc[a] = 0;

	int bestC[16], bestA[16];
	const int errC = ComputeSubsetTable(cfg, area, wc, 1 << s.colorBits, vc, bestC);
	const int errA = ComputeSubsetTable(cfg, area, wa, 1 << s.alphaBits, va, bestA);

	uint64_t idxC = 0, idxA = 0;
	for (uint32_t i = 0; i < area.count; i++)
	{
		idxC |= uint64_t(uint32_t(bestC[i])) << (area.idx[i] * s.colorBits);
		idxA |= uint64_t(uint32_t(bestA[i])) << (area.idx[i] * s.alphaBits);
	}
	int errorAlpha = 0;
	{
		const uint16_t(*vals)[4] = (a == 0) ? va : vc;
		const int* best = (a == 0) ? bestA : bestC;
		for (uint32_t i = 0; i < area.count; i++)
		{
			int da = int(vals[best[i]][0]) - int(area.px[i][0]);
			da = da < 0 ? -da : da;
			if (!cfg.denoise)
				da = da > 0x7F ? 0x7F : da;
			else
				da >>= cfg.denoise;
			errorAlpha += da * da;
		}
	}
	input.errAlpha = errorAlpha * cfg.wA;
	input.errTotal = errC + errA;

	V8 mcolor = mc, malpha = mc;
	if (s.colorBits == 3)
		AreaReduceTable3(area, mcolor, idxC);
	else
		AreaReduceTable2(area, mcolor, idxC);
	if (s.alphaBits == 3)
		AreaReduceTable3(area, malpha, idxA);
	else
		AreaReduceTable2(area, malpha, idxA);
	mc = mcolor;
	mc.l[0] = malpha.l[0];
	mc.l[1] = malpha.l[1];

	BitWriter bw;
	const int anchors[1] = { 0 };
	if (mode4)
	{
		bw.Put(16, 5);
		bw.Put(uint64_t(rotation & 3), 2);
		bw.Put(uint64_t((rotation >> 2) & 1), 1);
		const int ch[3] = { 2, 1, 3 };
		for (int c = 0; c < 3; c++)
			for (int k = 0; k < 2; k++)
				bw.Put(uint64_t((mc.l[2 * ch[c] + k] >> 3) & 0x1F), 5);
		for (int k = 0; k < 2; k++)
			bw.Put(uint64_t((mc.l[k] >> 2) & 0x3F), 6);
		/* 2-bit index set first, then the 3-bit one */
		if (s.colorBits == 2)
		{
			PutIndices(bw, idxC, 2, anchors, 1);
			PutIndices(bw, idxA, 3, anchors, 1);
		}
		else
		{
			PutIndices(bw, idxA, 2, anchors, 1);
			PutIndices(bw, idxC, 3, anchors, 1);
		}
	}
	else
	{
		bw.Put(32, 6);
		bw.Put(uint64_t(rotation & 3), 2);
		const int ch[3] = { 2, 1, 3 };
		for (int c = 0; c < 3; c++)
			for (int k = 0; k < 2; k++)
				bw.Put(uint64_t((mc.l[2 * ch[c] + k] >> 1) & 0x7F), 7);
		for (int k = 0; k < 2; k++)
			bw.Put(uint64_t(mc.l[k] & 0xFF), 8);
		PutIndices(bw, idxC, 2, anchors, 1);
		PutIndices(bw, idxA, 2, anchors, 1);
	}
	bw.Store(out);
}

} // namespace

namespace mode4 {

void FinalPack(const Config& cfg, uint8_t* out, Cell& input)
{
	FinalPackRot(cfg, out, input, true);
}

static int SubsetFast(const Config& cfg, const Area& area, uint8_t mcStorage[8], int water, int rotation)
{
	/* src/Bc7CoreMode4.cpp:1195-1223 */
	V8 b;
	memcpy(b.l, area.bounds, sizeof(b.l));
	uint8_t epI[8], epS[8];
	Pack(b, epI);
	SwapRot(epI, epS, rotation);
	for (int i = 0; i < 8; i++)
	{
		if (i < 2)
			epS[i] = uint8_t((epS[i] & 0xFC) | (epS[i] >> 6));
		else
			epS[i] = uint8_t((epS[i] & 0xF8) | (epS[i] >> 5));
	}
	memcpy(mcStorage, epS, 8);
	SwapRot(epS, epI, rotation);
	const RotSpec s = SpecFor(cfg, true, rotation);
	const int w[4] = { cfg.wA, cfg.wG, cfg.wR, cfg.wB };
	return RotError(cfg, area, epI, rotation, s.colorBits, s.alphaBits, w, water, true);
}

void Fast(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode4.cpp:1225-1255 */
	const int step = input.denoiseStep;
	for (int ri = 0; ri < 8; ri++)
	{
		const int rotation = kRotationsMode4[ri];
		uint8_t mc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
		int error = step;
		if (error < input.errTotal)
			error += SubsetFast(cfg, input.area1, mc, input.errTotal - error, rotation);
		if (input.errTotal > error)
		{
			input.errTotal = error - step;
			input.best0 = Widen(mc);
			input.bestParam = uint64_t(rotation);
			input.bestMode = 4;
			if (error <= step)
				break;
		}
	}
}

void Refine(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode4.cpp:1795-1822 */
	int rotation = int(input.bestParam);
	for (int i = 0; i < 2; i++, rotation ^= 4)
	{
		uint8_t mc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
		int error = 0;
		error += CompressRotSubset(cfg, true, input.area1, mc, input.errTotal - error, rotation);
		if (input.errTotal > error)
		{
			input.errTotal = error;
			input.best0 = Widen(mc);
			input.bestParam = uint64_t(rotation);
			if (error <= 0)
				break;
		}
	}
}

void Full(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode4.cpp:1824-1857 */
	const int step = input.denoiseStep;
	for (int ri = 0; ri < 8; ri++)
	{
		const int rotation = kRotationsMode4[ri];
		if (input.personalMode == 4 && !((input.personalParam ^ uint64_t(rotation)) & 3))
			continue;
		uint8_t mc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
		int error = step;
		if (error < input.errTotal)
			error += CompressRotSubset(cfg, true, input.area1, mc, input.errTotal - error, rotation);
		if (input.errTotal > error)
		{
			input.errTotal = error - step;
			input.best0 = Widen(mc);
			input.bestParam = uint64_t(rotation);
			input.bestMode = 4;
			if (error <= step)
				break;
		}
	}
}

} // namespace mode4

namespace mode5 {

void FinalPack(const Config& cfg, uint8_t* out, Cell& input)
{
	FinalPackRot(cfg, out, input, false);
}

static int SubsetFast(const Config& cfg, const Area& area, uint8_t mcStorage[8], int water, int rotation)
{
	/* src/Bc7CoreMode5.cpp:569-587 */
	V8 b;
	memcpy(b.l, area.bounds, sizeof(b.l));
	uint8_t epI[8], epS[8];
	Pack(b, epI);
	SwapRot(epI, epS, rotation);
	for (int i = 2; i < 8; i++)
		epS[i] = uint8_t((epS[i] & 0xFE) | (epS[i] >> 7));
	memcpy(mcStorage, epS, 8);
	SwapRot(epS, epI, rotation);
	const int w[4] = { cfg.wA, cfg.wG, cfg.wR, cfg.wB };
	return RotError(cfg, area, epI, rotation, 2, 2, w, water, false);
}

void Fast(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode5.cpp:589-619 */
	const int step = input.denoiseStep;
	for (int ri = 0; ri < 4; ri++)
	{
		const int rotation = kRotationsMode5[ri];
		uint8_t mc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
		int error = step;
		if (error < input.errTotal)
			error += SubsetFast(cfg, input.area1, mc, input.errTotal - error, rotation);
		if (input.errTotal > error)
		{
			input.errTotal = error - step;
			input.best0 = Widen(mc);
			input.bestParam = uint64_t(rotation);
			input.bestMode = 5;
			if (error <= step)
				break;
		}
	}
}

void Refine(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode5.cpp:890-911 */
	const int rotation = int(input.bestParam);
	uint8_t mc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
	int error = 0;
	error += CompressRotSubset(cfg, false, input.area1, mc, input.errTotal - error, rotation);
	if (input.errTotal > error)
	{
		input.errTotal = error;
		input.best0 = Widen(mc);
	}
}

void Full(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode5.cpp:913-946 */
	const int step = input.denoiseStep;
	for (int ri = 0; ri < 4; ri++)
	{
		const int rotation = kRotationsMode5[ri];
		if (input.personalMode == 5 && input.personalParam == uint64_t(rotation))
			continue;
		uint8_t mc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
		int error = step;
		if (error < input.errTotal)
			error += CompressRotSubset(cfg, false, input.area1, mc, input.errTotal - error, rotation);
		if (input.errTotal > error)
		{
			input.errTotal = error - step;
			input.best0 = Widen(mc);
			input.bestParam = uint64_t(rotation);
			input.bestMode = 5;
			if (error <= step)
				break;
		}
	}
}

} // namespace mode5

/* ======================================================================= */
/* Modes 6, 6Index2 and 7: four channels with a transparent-alpha term      */
/* ======================================================================= */
namespace {

struct Est4
{
	int ch0, ch1, ch2, ch3;
};

struct Rgba4Spec
{
	int indexBits;            /* 4 for mode 6, 2 for Mode6Index2 and mode 7 */
	bool half;                /* nibble tables (modes 6 / 6I2) */
	int bits;                 /* LevelsBuffer bits */
	const uint8_t* table;
	int maxSize;
	bool transparent4;        /* transparent error from the clamped 4-bit table */
};

struct Subset4
{
	Levels ch[4];

	/* src/Bc7CoreMode6.cpp:1130-1161, src/Bc7CoreMode6Index2.cpp:137-168,
	   src/Bc7CoreMode7.cpp:237-268 */
	bool InitLevels(const Config& cfg, const Rgba4Spec& s, int pbits, const Area& area, int water, const Est4& est)
	{
		for (int c = 0; c < 4; c++)
			LevelsInit(ch[c], cfg);
		const int wts[4] = { cfg.wA, cfg.wG, cfg.wR, cfg.wB };
		const int estv[4] = { est.ch0, est.ch1, est.ch2, est.ch3 };
		int used = 0;
		for (int c = 0; c < 4; c++)
		{
			int rest = 0;
			for (int k = c + 1; k < 4; k++)
				rest += estv[k];
			if (c == 0 && area.opaque)
			{
				ch[0].minErr = 0;
				ch[0].count = 1;
				ch[0].e[0].err = 0;
				ch[0].e[0].color = 0xFFFF;
			}
			else if (s.half)
			{
				ChannelLevelsHalf(cfg, ch[c], area, c, wts[c], water - used - rest, s.bits, pbits, c != 0, s.table, s.maxSize);
			}
			else
			{
				ChannelLevels(cfg, ch[c], area, c, wts[c], water - used - rest, s.bits, pbits, c != 0, s.table, false, s.maxSize);
			}
			used += ch[c].minErr;
			if (used >= water)
				return false;
		}
		return true;
	}

	int Transparent(const Config& cfg, const Rgba4Spec& s, const Area& area, int alpha) const
	{
		return s.transparent4 ? TransparentError4(cfg, area, alpha) : TransparentError2(cfg, area, alpha);
	}

	/* src/Bc7CoreMode6.cpp:1163-1331 (same in 6Index2 and 7) */
	int TryVariants(const Config& cfg, const Rgba4Spec& s, const Area& area, V8& best, int water)
	{
		const int min0 = ch[0].minErr, min1 = ch[1].minErr, min2 = ch[2].minErr, min3 = ch[3].minErr;
		if (min0 + min1 + min2 + min3 >= water)
			return water;
		const int n0 = ch[0].count, n1 = ch[1].count, n2 = ch[2].count, n3 = ch[3].count;
		const W4 wAG = Wt(cfg, true, true, false, false);
		const W4 wAR = Wt(cfg, true, false, true, false);
		const W4 wGR = Wt(cfg, false, true, true, false);
		const W4 wAGR = Wt(cfg, true, true, true, false);
		const W4 wGB = Wt(cfg, false, true, false, true);
		const W4 wAGB = Wt(cfg, true, true, false, true);
		const W4 wAGRB = Wt(cfg, true, true, true, true);
		const int ib = s.indexBits;
		int memAR[32], memAGB[32];

		for (int i0 = 0; i0 < n0; i0++)
		{
			const int e0 = ch[0].e[i0].err;
			if (e0 + min1 + min2 + min3 >= water)
				break;
			const int c0 = ch[0].e[i0].color;
			const int ea = Transparent(cfg, s, area, c0);
			for (int i = 0; i < n2; i++)
				memAR[i] = -1;
			for (int i1 = 0; i1 < n1; i1++)
			{
				int e1 = ch[1].e[i1].err + e0;
				if (e1 + min2 + min3 >= water)
					break;
				const int c1 = ch[1].e[i1].color;
				if (!area.opaque)
				{
					uint8_t ep[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
					SetCh(ep, 0, c0);
					SetCh(ep, 1, c1);
					e1 = SubsetError(cfg, area, ep, ib, wAG.w, water - ea - min2 - min3) + ea;
					if (e1 + min2 + min3 >= water)
						continue;
				}
				for (int i = 0; i < n3; i++)
					memAGB[i] = -1;
				for (int i2 = 0; i2 < n2; i2++)
				{
					int e2 = ch[2].e[i2].err + e1;
					if (e2 + min3 >= water)
						break;
					const int c2 = ch[2].e[i2].color;
					if (!area.opaque)
					{
						int ear = memAR[i2];
						if (ear < 0)
						{
							uint8_t ep[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
							SetCh(ep, 0, c0);
							SetCh(ep, 2, c2);
							ear = SubsetError(cfg, area, ep, ib, wAR.w, water - ea - min1 - min3) + ea;
							memAR[i2] = ear;
						}
						if (ear + min1 + min3 >= water)
							continue;
					}
					{
						uint8_t ep[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
						SetCh(ep, 0, c0);
						SetCh(ep, 1, c1);
						SetCh(ep, 2, c2);
						if (area.opaque)
							e2 = SubsetError(cfg, area, ep, ib, wGR.w, water - ea - min3) + ea;
						else
							e2 = SubsetError(cfg, area, ep, ib, wAGR.w, water - ea - min3) + ea;
						if (e2 + min3 >= water)
							continue;
					}
					for (int i3 = 0; i3 < n3; i3++)
					{
						const int e3 = ch[3].e[i3].err + e2;
						if (e3 >= water)
							break;
						const int c3 = ch[3].e[i3].color;
						int eagb = memAGB[i3];
						if (eagb < 0)
						{
							uint8_t ep[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
							SetCh(ep, 0, c0);
							SetCh(ep, 1, c1);
							SetCh(ep, 3, c3);
							if (area.opaque)
								eagb = SubsetError(cfg, area, ep, ib, wGB.w, water - ea - min2) + ea;
							else
								eagb = SubsetError(cfg, area, ep, ib, wAGB.w, water - ea - min2) + ea;
							memAGB[i3] = eagb;
						}
						if (eagb + min2 >= water)
							continue;
						uint8_t ep[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
						SetCh(ep, 0, c0);
						SetCh(ep, 1, c1);
						SetCh(ep, 2, c2);
						SetCh(ep, 3, c3);
						const int err = SubsetError(cfg, area, ep, ib, wAGRB.w, water - ea) + ea;
						if (water > err)
						{
							water = err;
							best = Widen(ep);
						}
					}
				}
			}
		}
		return water;
	}
};

const Est4 kNoEst = { 0, 0, 0, 0 };

/* Mode 6 / 6Index2 CompressSubset (src/Bc7CoreMode6.cpp:1334-1364): each
   later p-bit variant starts from the water left by the earlier ones. */
int CompressSubsetSingle(const Config& cfg, const Rgba4Spec& s, const Area& area, V8& mc, int water)
{
	{
		Subset4 sub;
		if (sub.InitLevels(cfg, s, 0x0101, area, water, kNoEst))
			water = sub.TryVariants(cfg, s, area, mc, water);
	}
	if (!area.opaque)
	{
		const int variants[3] = { 0, 1, 1 << 8 };
		for (int v = 0; v < 3; v++)
		{
			Subset4 sub;
			if (sub.InitLevels(cfg, s, variants[v], area, water, kNoEst))
				water = sub.TryVariants(cfg, s, area, mc, water);
		}
	}
	return water;
}

Rgba4Spec Spec6(const Config& cfg) { return Rgba4Spec{ 4, true, 7, cfg.lt->d4h, 20, true }; }
Rgba4Spec Spec6i2(const Config& cfg) { return Rgba4Spec{ 2, true, 7, cfg.lt->d2h, 20, false }; }
Rgba4Spec Spec7(const Config& cfg) { return Rgba4Spec{ 2, false, 5, cfg.lt->d2v6, 20, false }; }

void ComposeMode6(uint8_t* out, const V8& mc, uint64_t indices)
{
	/* src/Bc7CoreMode6.cpp:89-115 */
	BitWriter bw;
	bw.Put(64, 7);
	const int ch[4] = { 2, 1, 3, 0 };
	for (int c = 0; c < 4; c++)
		for (int k = 0; k < 2; k++)
			bw.Put(uint64_t((mc.l[2 * ch[c] + k] >> 1) & 0x7F), 7);
	bw.Put(uint64_t(mc.l[0] & 1), 1);
	bw.Put(uint64_t(mc.l[1] & 1), 1);
	const int anchors[1] = { 0 };
	PutIndices(bw, indices, 4, anchors, 1);
	bw.Store(out);
}

} // namespace

namespace mode6 {

void FinalPack(const Config& cfg, uint8_t* out, Cell& input)
{
	/* src/Bc7CoreMode6.cpp:933-1075 */
	Area& area = input.area1;
	V8 mc = input.best0;
	uint8_t ep[8];
	Pack(mc, ep);
	uint16_t vals[16][4];
	InterpolateLevels(ep, 4, vals);
	const int w[4] = { cfg.wA, cfg.wG, cfg.wR, cfg.wB };
	int best[16];
	const int error = ComputeSubsetTable(cfg, area, w, 16, vals, best);
	uint64_t indices = 0;
	for (int i = 0; i < 16; i++)
		indices |= uint64_t(uint32_t(best[i])) << (area.idx[i] << 2);
	int errorAlpha = 0;
	for (int i = 0; i < 16; i++)
	{
		int da = int(vals[best[i]][0]) - int(area.px[i][0]);
		da = da < 0 ? -da : da;
		if (!cfg.denoise)
			da = da > 0x7F ? 0x7F : da;
		else
			da >>= cfg.denoise;
		errorAlpha += da * da;
	}
	input.errAlpha = errorAlpha * cfg.wA;
	input.errTotal = error;
	AreaReduceTable4(mc, indices);
	ComposeMode6(out, mc, indices);
}

static int SubsetFast(const Config& cfg, const Area& area, V8& mc, int water)
{
	/* src/Bc7CoreMode6.cpp:1077-1098 */
	V8 m;
	memcpy(m.l, area.bounds, sizeof(m.l));
	const int p0 = m.l[0] & 1, p1 = m.l[1] & 1;
	for (int i = 0; i < 8; i++)
		m.l[i] = int16_t((m.l[i] & 0xFE) | ((i & 1) ? p1 : p0));
	mc = m;
	uint8_t ep[8];
	Pack(mc, ep);
	const int ea = TransparentError4(cfg, area, PackedAlpha(ep));
	if (ea >= water)
		return water;
	const int w[4] = { cfg.wA, cfg.wG, cfg.wR, cfg.wB };
	return SubsetError(cfg, area, ep, 4, w, water - ea) + ea;
}

void Fast(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode6.cpp:1100-1121 */
	const int step = input.denoiseStep;
	V8 mc = V8Zero();
	int error = step;
	if (error < input.errTotal)
		error += SubsetFast(cfg, input.area1, mc, input.errTotal - error);
	if (input.errTotal > error)
	{
		input.errTotal = error - step;
		input.best0 = mc;
		input.bestMode = 6;
	}
}

void Refine(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode6.cpp:1366-1381 */
	V8 mc = input.best0;
	const int error = CompressSubsetSingle(cfg, Spec6(cfg), input.area1, mc, input.errTotal);
	if (input.errTotal > error)
	{
		input.errTotal = error;
		input.best0 = mc;
	}
}

void Full(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode6.cpp:1398-1422 */
	if (input.personalMode == 6)
		return;
	const int step = input.denoiseStep;
	/* EstimateBest (src/Bc7CoreMode6.cpp:1383-1396): 0 without OPTION_PCA */
	const int line = cfg.pca ? PcaBound(cfg, input.area1, input.area1.opaque ? 3 : 4) : 0;
	if (line < input.errTotal - step)
	{
		V8 mc = V8Zero();
		const int error = CompressSubsetSingle(cfg, Spec6(cfg), input.area1, mc, input.errTotal - step);
		if (input.errTotal > error + step)
		{
			input.errTotal = error;
			input.best0 = mc;
			input.bestMode = 6;
		}
	}
}

} // namespace mode6

namespace mode6i2 {

void FinalPack(const Config& cfg, uint8_t* out, Cell& input)
{
	/* src/Bc7CoreMode6Index2.cpp:62-82 */
	Area& area = input.area1;
	V8 mc = input.best0;
	uint64_t indices2 = 0;
	int errorAlpha = 0;
	const int error = OpaqueTable(cfg, area, mc, 2, indices2, false, &errorAlpha);
	input.errAlpha = errorAlpha;
	input.errTotal = error;
	uint64_t indices = 0;
	for (uint32_t i = 0; i < area.count; i++)
	{
		uint64_t index = (indices2 >> (i << 1)) & 3u;
		index += index << 2;
		indices |= index << (i << 2);
	}
	AreaReduceTable4(mc, indices);
	ComposeMode6(out, mc, indices);
}

static int SubsetFast(const Config& cfg, const Area& area, V8& mc, int water)
{
	/* src/Bc7CoreMode6Index2.cpp:84-105 */
	V8 m;
	memcpy(m.l, area.bounds, sizeof(m.l));
	const int p0 = m.l[0] & 1, p1 = m.l[1] & 1;
	for (int i = 0; i < 8; i++)
		m.l[i] = int16_t((m.l[i] & 0xFE) | ((i & 1) ? p1 : p0));
	mc = m;
	uint8_t ep[8];
	Pack(mc, ep);
	const int ea = TransparentError2(cfg, area, PackedAlpha(ep));
	if (ea >= water)
		return water;
	const int w[4] = { cfg.wA, cfg.wG, cfg.wR, cfg.wB };
	return SubsetError(cfg, area, ep, 2, w, water - ea) + ea;
}

void Fast(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode6Index2.cpp:107-128 */
	const int step = input.denoiseStep;
	V8 mc = V8Zero();
	int error = step;
	if (error < input.errTotal)
		error += SubsetFast(cfg, input.area1, mc, input.errTotal - error);
	if (input.errTotal > error)
	{
		input.errTotal = error - step;
		input.best0 = mc;
		input.bestMode = 9;
	}
}

void Refine(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode6Index2.cpp:373-388 */
	V8 mc = input.best0;
	const int error = CompressSubsetSingle(cfg, Spec6i2(cfg), input.area1, mc, input.errTotal);
	if (input.errTotal > error)
	{
		input.errTotal = error;
		input.best0 = mc;
	}
}

} // namespace mode6i2

namespace mode7 {

void FinalPack(const Config& cfg, uint8_t* out, Cell& input)
{
	/* src/Bc7CoreMode7.cpp:85-159 */
	const Selection& sel = *cfg.sel;
	const int p = int(input.bestParam);
	Area& a1 = GetArea(cfg, input.a12[p], input.lazy12[p], input, sel.sel12[p]);
	Area& a2 = GetArea(cfg, input.a22[p], input.lazy22[p], input, sel.sel22[p]);
	V8 mc0 = input.best0, mc1 = input.best1;
	uint64_t indices = 0;
	int ea0 = 0, ea1 = 0;
	const int e0 = OpaqueTable(cfg, a1, mc0, 2, indices, false, &ea0);
	const int e1 = OpaqueTable(cfg, a2, mc1, 2, indices, false, &ea1);
	input.errAlpha = ea0 + ea1;
	input.errTotal = e0 + e1;
	AreaReduceTable2(a1, mc0, indices);
	AreaReduceTable2(a2, mc1, indices);

	const V8* mc[2] = { &mc0, &mc1 };
	BitWriter bw;
	bw.Put(128, 8);
	bw.Put(uint64_t(p), 6);
	const int ch[4] = { 2, 1, 3, 0 };
	for (int c = 0; c < 4; c++)
		for (int s = 0; s < 2; s++)
			for (int k = 0; k < 2; k++)
				bw.Put(uint64_t((mc[s]->l[2 * ch[c] + k] >> 3) & 0x1F), 5);
	for (int s = 0; s < 2; s++)
		for (int k = 0; k < 2; k++)
			bw.Put(uint64_t((mc[s]->l[k] >> 2) & 1), 1);
	const int anchors[2] = { 0, kAnchor2of2[p] };
	PutIndices(bw, indices, 2, anchors, 2);
	bw.Store(out);
}

static int SubsetFast(const Config& cfg, const Area& area, V8& mc, int water)
{
	/* src/Bc7CoreMode7.cpp:161-184 */
	V8 m;
	memcpy(m.l, area.bounds, sizeof(m.l));
	const int p0 = m.l[0] & 4, p1 = m.l[1] & 4;
	for (int i = 0; i < 8; i++)
	{
		int v = m.l[i] & 0xF8;
		v |= v >> 6;
		v |= (i & 1) ? p1 : p0;
		m.l[i] = int16_t(v);
	}
	mc = m;
	uint8_t ep[8];
	Pack(mc, ep);
	const int ea = TransparentError2(cfg, area, PackedAlpha(ep));
	if (ea >= water)
		return water;
	const int w[4] = { cfg.wA, cfg.wG, cfg.wR, cfg.wB };
	return SubsetError(cfg, area, ep, 2, w, water - ea) + ea;
}

void Fast(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode7.cpp:186-223 */
	const int step = input.denoiseStep;
	const Selection& sel = *cfg.sel;
	for (int p = 0; p < 64; p++)
	{
		V8 mc0 = V8Zero(), mc1 = V8Zero();
		int error = step;
		if (error < input.errTotal)
		{
			Area& a1 = GetArea(cfg, input.a12[p], input.lazy12[p], input, sel.sel12[p]);
			error += SubsetFast(cfg, a1, mc0, input.errTotal - error);
			if (error < input.errTotal)
			{
				Area& a2 = GetArea(cfg, input.a22[p], input.lazy22[p], input, sel.sel22[p]);
				error += SubsetFast(cfg, a2, mc1, input.errTotal - error);
				if (input.errTotal > error)
				{
					input.errTotal = error - step;
					input.best0 = mc0;
					input.best1 = mc1;
					input.bestParam = uint64_t(p);
					input.bestMode = 7;
					if (error <= step)
						return;
				}
			}
		}
	}
}

/* src/Bc7CoreMode7.cpp:441-494: variants' lists all start from the same water. */
struct Subsets7
{
	Subset4 sub[4];
	bool valid[4];

	bool InitLevels(const Config& cfg, const Rgba4Spec& s, const Area& area, int water, const Est4& est)
	{
		const int pb[4] = { 0x0101, 0, 1, 1 << 8 };
		valid[0] = sub[0].InitLevels(cfg, s, pb[0], area, water, est);
		valid[1] = valid[2] = valid[3] = false;
		if (!area.opaque)
			for (int v = 1; v < 4; v++)
				valid[v] = sub[v].InitLevels(cfg, s, pb[v], area, water, est);
		return valid[0] || valid[1] || valid[2] || valid[3];
	}

	int TryVariants(const Config& cfg, const Rgba4Spec& s, const Area& area, V8& best, int water)
	{
		for (int v = 0; v < 4; v++)
			if (valid[v])
				water = sub[v].TryVariants(cfg, s, area, best, water);
		return water;
	}
};

void Refine(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode7.cpp:496-557 */
	const Selection& sel = *cfg.sel;
	const int p = int(input.bestParam);
	V8 mc[2] = { input.best0, input.best1 };
	const Rgba4Spec s = Spec7(cfg);
	const int w[4] = { cfg.wA, cfg.wG, cfg.wR, cfg.wB };

	int error = 0;
	for (int si = 0; si < 2; si++)
	{
		Area& area = si == 0 ? GetArea(cfg, input.a12[p], input.lazy12[p], input, sel.sel12[p])
			: GetArea(cfg, input.a22[p], input.lazy22[p], input, sel.sel22[p]);
		uint8_t ep[8];
		Pack(mc[si], ep);
		int water = SubsetError(cfg, area, ep, 2, w, cfg.MaxColorAlphaError());
		water += TransparentError2(cfg, area, PackedAlpha(ep));
		if (water)
		{
			Subsets7 subs;
			if (subs.InitLevels(cfg, s, area, water, kNoEst))
				error += subs.TryVariants(cfg, s, area, mc[si], water);
			else
				error += water;
		}
	}
	if (input.errTotal > error)
	{
		input.errTotal = error;
		input.best0 = mc[0];
		input.best1 = mc[1];
	}
}

static int EstimateLevels(const Config& cfg, const Area& area, int water, Est4& est)
{
	/* src/Bc7CoreMode7.cpp:574-627 */
	int error = 0;
	if (error < water)
	{
		if (!area.active)
		{
			est.ch0 = est.ch1 = est.ch2 = est.ch3 = 0;
			return 0;
		}
		if (!area.opaque)
		{
			const int l0 = EstimateChannelLevels(cfg, area, 0, cfg.wA, water - error, 6, false, cfg.lt->d2v6, cfg.lt->c2v6);
			est.ch0 = l0;
			error += l0;
		}
		else
		{
			est.ch0 = 0;
		}
		if (error < water)
		{
			const int l1 = EstimateChannelLevels(cfg, area, 1, cfg.wG, water - error, 6, true, cfg.lt->d2v6, cfg.lt->c2v6);
			est.ch1 = l1;
			error += l1;
			if (error < water)
			{
				const int l2 = EstimateChannelLevels(cfg, area, 2, cfg.wR, water - error, 6, true, cfg.lt->d2v6, cfg.lt->c2v6);
				est.ch2 = l2;
				error += l2;
				if (error < water)
				{
					const int l3 = EstimateChannelLevels(cfg, area, 3, cfg.wB, water - error, 6, true, cfg.lt->d2v6, cfg.lt->c2v6);
					est.ch3 = l3;
					error += l3;
					if (error < water)
						return error;
				}
			}
		}
	}
	return water;
}

void Full(const Config& cfg, Cell& input)
{
	/* src/Bc7CoreMode7.cpp:629-725 */
	Node order[64];
	int lines1[64], lines2[64];
	const int step = input.denoiseStep;
	const Selection& sel = *cfg.sel;
	const Rgba4Spec s = Spec7(cfg);

	int count = 0;
	for (int p = 0; p < 64; p++)
	{
		if (input.personalMode == 7 && input.personalParam == uint64_t(p))
			continue;
		GetArea(cfg, input.a12[p], input.lazy12[p], input, sel.sel12[p]);
		const int water1 = input.errTotal - step;
		/* EstimateBest (src/Bc7CoreMode7.cpp:559-572): 0 without OPTION_PCA */
		const int line1 = cfg.pca ? PcaBound(cfg, input.a12[p], input.a12[p].opaque ? 3 : 4) : 0;
		if (line1 < water1)
		{
			GetArea(cfg, input.a22[p], input.lazy22[p], input, sel.sel22[p]);
			const int water2 = water1 - line1;
			const int line2 = cfg.pca ? PcaBound(cfg, input.a22[p], input.a22[p].opaque ? 3 : 4) : 0;
			if (line2 < water2)
			{
				lines1[p] = line1;
				lines2[p] = line2;
				order[count].err = line1 + line2 + step;
				order[count].color = p;
				count++;
			}
		}
	}

	RadixSortPartitions(order, count);

	for (int i = 0; i < count; i++)
	{
		if (order[i].err < input.errTotal)
		{
			const int p = order[i].color;
			V8 mc0 = V8Zero(), mc1 = V8Zero();
			Area& area1 = GetArea(cfg, input.a12[p], input.lazy12[p], input, sel.sel12[p]);
			Area& area2 = GetArea(cfg, input.a22[p], input.lazy22[p], input, sel.sel22[p]);
			int line1 = lines1[p];
			int line2 = lines2[p];
			Est4 e1, e2;
			int water1 = input.errTotal - step - line2;
			{
				const int l = EstimateLevels(cfg, area1, water1, e1);
				line1 = line1 > l ? line1 : l;
			}
			if (line1 < water1)
			{
				int water2 = water1 - line1;
				{
					const int l = EstimateLevels(cfg, area2, water2, e2);
					line2 = line2 > l ? line2 : l;
				}
				if (line2 < water2)
				{
					water1 = input.errTotal - step - line2;
					Subsets7 subs1;
					if (subs1.InitLevels(cfg, s, area1, water1, e1))
					{
						int error = subs1.TryVariants(cfg, s, area1, mc0, water1);
						if (error < water1)
						{
							water2 = input.errTotal - step - error;
							Subsets7 subs2;
							if (subs2.InitLevels(cfg, s, area2, water2, e2))
							{
								error += subs2.TryVariants(cfg, s, area2, mc1, water2);
								if (input.errTotal > error + step)
								{
									input.errTotal = error;
									input.best0 = mc0;
									input.best1 = mc1;
									input.bestParam = uint64_t(p);
									input.bestMode = 7;
									if (error <= 0)
										return;
								}
							}
						}
					}
				}
			}
		}
	}
}

} // namespace mode7

} // namespace nebc7_oracle
