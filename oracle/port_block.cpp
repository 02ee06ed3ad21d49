/*
 * CPU oracle for the BC7 block encoder -- BPTC block layout and the
 * per-block scheduler (test infrastructure only; see port_tables.h).
 *
 * Decoders restate src/Bc7CoreMode{0..7}.cpp DecompressBlock and
 * src/Bc7Core.cpp:1446; the scheduler restates src/Bc7Core.cpp:24-109 and
 * 1516-1823 (CompressBlock).
 */
#include "port_core.h"

#include <string.h>

namespace nebc7_oracle {

namespace {

struct BitReader
{
	uint64_t lo, hi;
	int pos;

	explicit BitReader(const uint8_t b[16])
	{
		memcpy(&lo, b, 8);
		memcpy(&hi, b + 8, 8);
		pos = 0;
	}

	int Get(int n)
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

inline int Expand(int v, int bits)
{
	/* bit replication to 8 bits */
	v <<= (8 - bits);
	return v | (v >> bits);
}

inline int Interp(int e0, int e1, int w)
{
	return (e0 * (64 - w) + e1 * w + 32) >> 6;
}

/* Reads per-pixel indices with one implicit zero MSB at each anchor. */
void ReadIndices(BitReader& br, int bits, const int* anchors, int nanchors, int out[16])
{
	for (int i = 0; i < 16; i++)
	{
		bool anchor = false;
		for (int a = 0; a < nanchors; a++)
			anchor |= anchors[a] == i;
		out[i] = br.Get(anchor ? bits - 1 : bits);
	}
}

void SetLanes(V8& v, int c, int e0, int e1)
{
	v.l[2 * c] = int16_t(e0);
	v.l[2 * c + 1] = int16_t(e1);
}

} // namespace

void DecompressBlock(const uint8_t block[16], Cell& out)
{
	const int encoded = block[0];
	int mode = 8;
	for (int m = 0; m < 8; m++)
	{
		if (encoded & (1 << m))
		{
			mode = m;
			break;
		}
	}

	out.best0 = V8Zero();
	out.best1 = V8Zero();
	out.best2 = V8Zero();
	out.bestParam = 0;
	out.bestMode = uint32_t(mode);

	if (mode == 8)
	{
		/* src/Bc7Core.cpp:1499-1513 */
		memset(out.img, 0, sizeof(out.img));
		return;
	}

	BitReader br(block);
	br.Get(mode + 1);

	const Selection& sel = GetSelection();

	if (mode == 0 || mode == 1 || mode == 2 || mode == 3 || mode == 7)
	{
		const int ns = (mode == 0 || mode == 2) ? 3 : 2;
		const int partition = br.Get(mode == 0 ? 4 : 6);
		const int cbits = mode == 0 ? 4 : (mode == 1 ? 6 : (mode == 2 ? 5 : (mode == 3 ? 7 : 5)));
		const bool hasAlpha = mode == 7;
		int e[3][2][4];  /* subset, endpoint, channel AGRB */
		const int order[3] = { 2, 1, 3 };  /* R, G, B fields */
		for (int oc = 0; oc < 3; oc++)
			for (int s = 0; s < ns; s++)
				for (int k = 0; k < 2; k++)
					e[s][k][order[oc]] = br.Get(cbits);
		if (hasAlpha)
			for (int s = 0; s < ns; s++)
				for (int k = 0; k < 2; k++)
					e[s][k][0] = br.Get(cbits);
		int p[3][2] = { { 0, 0 }, { 0, 0 }, { 0, 0 } };
		bool hasP = (mode != 2);
		if (mode == 1)
		{
			for (int s = 0; s < ns; s++)
			{
				p[s][0] = p[s][1] = br.Get(1);
			}
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
		int anchors[3];
		int nanchors;
		if (ns == 3)
		{
			anchors[0] = 0;
			anchors[1] = kAnchor2of3[partition];
			anchors[2] = kAnchor3of3[partition];
			nanchors = 3;
		}
		else
		{
			anchors[0] = 0;
			anchors[1] = kAnchor2of2[partition];
			nanchors = 2;
		}
		int idx[16];
		ReadIndices(br, ibits, anchors, nanchors, idx);
		const int* w = ibits == 3 ? kInterp3 : kInterp2;
		for (int i = 0; i < 16; i++)
		{
			const int s = ns == 3 ? int((kPartition3[partition] >> (2 * i)) & 3) : int((kPartition2[partition] >> (2 * i)) & 3);
			for (int c = 0; c < 4; c++)
				out.img[i][c] = uint8_t(Interp(ex[s][0][c], ex[s][1][c], w[idx[i]]));
		}
		V8* bc[3] = { &out.best0, &out.best1, &out.best2 };
		for (int s = 0; s < ns; s++)
			for (int c = 0; c < 4; c++)
				SetLanes(*bc[s], c, ex[s][0][c], ex[s][1][c]);
		out.bestParam = uint64_t(partition);
		(void)sel;
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
		int idxA[16], idxB[16];
		const int anchors[1] = { 0 };
		int colorBits, alphaBits;
		if (mode == 4)
		{
			ReadIndices(br, 2, anchors, 1, idxA);  /* primary, 2-bit */
			ReadIndices(br, 3, anchors, 1, idxB);  /* secondary, 3-bit */
			colorBits = idxMode ? 3 : 2;
			alphaBits = idxMode ? 2 : 3;
		}
		else
		{
			ReadIndices(br, 2, anchors, 1, idxA);
			ReadIndices(br, 2, anchors, 1, idxB);
			colorBits = 2;
			alphaBits = 2;
		}
		for (int i = 0; i < 16; i++)
		{
			int ci, ai;
			if (mode == 4)
			{
				ci = idxMode ? idxB[i] : idxA[i];
				ai = idxMode ? idxA[i] : idxB[i];
			}
			else
			{
				ci = idxA[i];
				ai = idxB[i];
			}
			const int* wc = colorBits == 3 ? kInterp3 : kInterp2;
			const int* wa = alphaBits == 3 ? kInterp3 : kInterp2;
			int v[4];
			v[0] = Interp(ex[0][0], ex[1][0], wa[ai]);
			for (int c = 1; c < 4; c++)
				v[c] = Interp(ex[0][c], ex[1][c], wc[ci]);
			/* rotation swaps A with R, G or B */
			if (rotation == 1)
			{
				int t = v[0]; v[0] = v[2]; v[2] = t;
			}
			else if (rotation == 2)
			{
				int t = v[0]; v[0] = v[1]; v[1] = t;
			}
			else if (rotation == 3)
			{
				int t = v[0]; v[0] = v[3]; v[3] = t;
			}
			for (int c = 0; c < 4; c++)
				out.img[i][c] = uint8_t(v[c]);
		}
		for (int c = 0; c < 4; c++)
			SetLanes(out.best0, c, ex[0][c], ex[1][c]);
		out.bestParam = uint64_t(rotation | (idxMode << 2));
		return;
	}

	/* mode 6 */
	{
		int e[2][4];
		const int order[4] = { 2, 1, 3, 0 };
		for (int oc = 0; oc < 4; oc++)
			for (int k = 0; k < 2; k++)
				e[k][order[oc]] = br.Get(7);
		int p0 = br.Get(1), p1 = br.Get(1);
		int ex[2][4];
		for (int c = 0; c < 4; c++)
		{
			ex[0][c] = (e[0][c] << 1) | p0;
			ex[1][c] = (e[1][c] << 1) | p1;
		}
		const int anchors[1] = { 0 };
		int idx[16];
		ReadIndices(br, 4, anchors, 1, idx);
		for (int i = 0; i < 16; i++)
			for (int c = 0; c < 4; c++)
				out.img[i][c] = uint8_t(Interp(ex[0][c], ex[1][c], kInterp4[idx[i]]));
		for (int c = 0; c < 4; c++)
			SetLanes(out.best0, c, ex[0][c], ex[1][c]);
		out.bestParam = 0;
	}
}

/* ---------------------------------------------------------------------- */
/* Scheduler                                                              */
/* ---------------------------------------------------------------------- */

/* src/Bc7Core.cpp:24-50 */
static int ComputeOpaqueAlphaError(const Config& cfg, const Area& area)
{
	int error = 0;
	if (!area.opaque)
	{
		for (uint32_t i = 0; i < area.count; i++)
		{
			int da = int(int16_t(area.px[i][0])) ^ 255;
			if (!cfg.denoise)
				da = (da > 0x7F) ? 0x7F : da;
			else
				da >>= cfg.denoise;
			error += da * da;
		}
		error *= cfg.wA;
	}
	return error;
}

/* src/Bc7Core.cpp:52-109 */
static void MakeCell(Cell& input, const Cell& decoded)
{
	input.best0 = decoded.best0;
	input.best1 = decoded.best1;
	input.best2 = decoded.best2;
	input.bestParam = decoded.bestParam;
	input.bestMode = decoded.bestMode;

	int flags = 0;
	int m0 = 255;
	for (int i = 0; i < 16; i++)
	{
		for (int c = 0; c < 4; c++)
		{
			/* _mm_cvtepi8_epi16 of the mask byte: 0xFF -> 0xFFFF */
			const uint16_t m = uint16_t(int16_t(int8_t(input.msk[i][c])));
			const uint16_t v = uint16_t(input.img[i][c] & m);
			input.px[i][c] = v;
			input.mk[i][c] = m;
		}
		/* bit i of the widened G mask, :72-76 */
		flags |= ((input.mk[i][1] >> i) & 1) << i;
		m0 &= input.px[i][0];
	}
	input.visibleFlags = flags;
	input.opaque = (m0 == 255);

	for (int p = 0; p < 64; p++)
	{
		input.lazy12[p] = true;
		input.lazy22[p] = true;
		input.lazy13[p] = true;
		input.lazy23[p] = true;
		input.lazy33[p] = true;
	}
}

void CompressBlock(const Config& cfg, uint8_t output[16], Cell& input)
{
	if (!output[0])
	{
		memset(output, 0, 16);
		output[0] = 1 << 6;
	}

	uint8_t saved[16];
	memcpy(saved, output, 16);

	Cell temp;
	DecompressBlock(output, temp);

	CompareBlocks(cfg, input, temp, input.errAlpha, input.errTotal);
	if (input.errTotal > 0)
	{
		MakeCell(input, temp);
		MakeAreaFromCell(cfg, input.area1, input, 16, 0xFEDCBA9876543210uLL);

		if (cfg.doDraft)
		{
			const int denoiseStep = int(input.area1.active) * ((cfg.denoiseStep * (input.area1.opaque ? cfg.wColor : cfg.wColorAlpha)) >> (cfg.denoise + cfg.denoise));
			input.denoiseStep = denoiseStep;
			input.opaqueAlphaError = ComputeOpaqueAlphaError(cfg, input.area1);

			const int water = input.errTotal;

			if (cfg.mode6Index2Only)
			{
				/* the "Mode6Index2 fast" run: the draft chain reduced to its
				   first pass (no counterpart in the reference) */
				if (input.errTotal > denoiseStep && (cfg.denoise > 0 || cfg.denoiseStep > 0))
					mode6i2::Fast(cfg, input);
			}
			else if (input.errTotal > denoiseStep)
			{
				if (cfg.denoise > 0 || cfg.denoiseStep > 0)
					mode6i2::Fast(cfg, input);
				if (input.errTotal > denoiseStep)
				{
					mode6::Fast(cfg, input);
					if (input.errTotal > denoiseStep)
					{
						mode4::Fast(cfg, input);
						if (input.errTotal > denoiseStep)
						{
							mode5::Fast(cfg, input);
							if (input.errTotal > denoiseStep)
								mode7::Fast(cfg, input);
						}
					}
				}
			}

			if (!cfg.mode6Index2Only && int16_t(input.area1.minmax[0]) > (255 - 16))
			{
				const int gate = input.opaqueAlphaError + denoiseStep;
				if (input.errTotal > gate)
				{
					mode3::Fast(cfg, input);
					if (input.errTotal > gate)
					{
						mode1::Fast(cfg, input);
						if (input.errTotal > gate)
						{
							mode2::Fast(cfg, input);
							if (input.errTotal > gate)
								mode0::Fast(cfg, input);
						}
					}
				}
			}

			if (cfg.doNormal && !cfg.mode6Index2Only)
			{
				switch (input.bestMode)
				{
				case 0: if (input.errTotal > input.opaqueAlphaError) mode0::Refine(cfg, input); break;
				case 1: if (input.errTotal > input.opaqueAlphaError) mode1::Refine(cfg, input); break;
				case 2: if (input.errTotal > input.opaqueAlphaError) mode2::Refine(cfg, input); break;
				case 3: if (input.errTotal > input.opaqueAlphaError) mode3::Refine(cfg, input); break;
				case 4: if (input.errTotal > 0) mode4::Refine(cfg, input); break;
				case 5: if (input.errTotal > 0) mode5::Refine(cfg, input); break;
				case 6: if (input.errTotal > 0) mode6::Refine(cfg, input); break;
				case 7: if (input.errTotal > 0) mode7::Refine(cfg, input); break;
				case 9: if (input.errTotal > 0) mode6i2::Refine(cfg, input); break;
				}

				input.personalParam = input.bestParam;
				input.personalMode = input.bestMode;

				if (input.area1.opaque)
				{
					const int gate = input.opaqueAlphaError + denoiseStep;
					if (input.errTotal > gate)
					{
						mode2::Full(cfg, input);
						if (input.errTotal > input.opaqueAlphaError + denoiseStep)
						{
							mode0::Full(cfg, input);
							if (cfg.doSlow)
							{
								if (input.errTotal > input.opaqueAlphaError + denoiseStep)
								{
									mode1::Full(cfg, input);
									if (input.errTotal > input.opaqueAlphaError + denoiseStep)
									{
										mode3::Full(cfg, input);
										if (input.errTotal > denoiseStep)
										{
											mode5::Full(cfg, input);
											if (input.errTotal > denoiseStep)
											{
												mode4::Full(cfg, input);
												if (input.errTotal > denoiseStep)
												{
													mode7::Full(cfg, input);
													if (input.errTotal > denoiseStep)
														mode6::Full(cfg, input);
												}
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
					if (input.errTotal > denoiseStep)
					{
						mode5::Full(cfg, input);
						if (input.errTotal > denoiseStep)
						{
							mode4::Full(cfg, input);
							if (input.errTotal > denoiseStep)
							{
								mode7::Full(cfg, input);
								if (cfg.doSlow)
								{
									if (input.errTotal > denoiseStep)
										mode6::Full(cfg, input);
								}
							}
						}
					}
				}
			}

			if (water > input.errTotal)
			{
				switch (input.bestMode)
				{
				case 0: mode0::FinalPack(cfg, output, input); break;
				case 1: mode1::FinalPack(cfg, output, input); break;
				case 2: mode2::FinalPack(cfg, output, input); break;
				case 3: mode3::FinalPack(cfg, output, input); break;
				case 4: mode4::FinalPack(cfg, output, input); break;
				case 5: mode5::FinalPack(cfg, output, input); break;
				case 6: mode6::FinalPack(cfg, output, input); break;
				case 7: mode7::FinalPack(cfg, output, input); break;
				case 9: mode6i2::FinalPack(cfg, output, input); break;
				}
				DecompressBlock(output, temp);
			}
		}

		/* self-check, src/Bc7Core.cpp:1799-1807 */
		DecompressBlock(output, temp);
		int ea, et;
		CompareBlocks(cfg, input, temp, ea, et);
		if (ea != input.errAlpha || et != input.errTotal)
			memcpy(output, saved, 16);

		CompareBlocksSSIM(cfg, input, temp, input.qualityAlpha, input.qualityColor);
	}
	else
	{
		input.qualityAlpha = 1.0;
		input.qualityColor = 1.0;
	}
}

} // namespace nebc7_oracle
