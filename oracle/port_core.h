/*
 * CPU oracle for the BC7 block encoder -- per-block state and primitives
 * (test infrastructure only; see port_tables.h).
 *
 * Restates reference src/Bc7Core.h (Area, Cell, Node, Modulations) and the
 * search primitives of src/Bc7Core.cpp and src/Snippet*.h in scalar C++.
 * A "V8" holds the eight 16-bit lanes the reference keeps in one __m128i:
 * endpoint vectors are laid out A0 A1 G0 G1 R0 R1 B0 B1 (lane 2c = endpoint
 * 0 of channel c, lane 2c+1 = endpoint 1), image channels in A,G,R,B order.
 */
#pragma once

#include "port_tables.h"

#include <stdint.h>

namespace nebc7_oracle {

struct V8
{
	int16_t l[8];
};

static inline V8 V8Zero()
{
	V8 v;
	for (int i = 0; i < 8; i++)
		v.l[i] = 0;
	return v;
}

/* Encoder configuration: the reference's compile-time preset
   (src/Bc7Mode.h:10-15) plus the InitTables flags and weights
   (src/Bc7Core.cpp:1877, src/Bc7Tables.cpp:789). */
struct Config
{
	int denoise;       /* kDenoise: 0 or 1 */
	int denoiseStep;   /* kDenoiseStep: 0 or 9 */
	bool doDraft, doNormal, doSlow;
	bool mode6Index2Only;   /* draft chain reduced to Mode6Index2 (no counterpart in the reference) */
	bool pca;               /* OPTION_PCA: the principal-axis bounds of the full searches */
	int wA, wG, wR, wB, wColor, wColorAlpha;
	const LevelTables* lt;
	const Selection* sel;

	int MaxColorError() const { return 16 * (255 >> denoise) * (255 >> denoise) * 1000 + 1; }
	int MaxColorAlphaError() const { return MaxColorError() * 2; }
	int Q(int d) const
	{
		d = d < 0 ? -d : d;
		if (denoise)
			return d >> denoise;
		return d > 127 ? 127 : d;
	}
};

void MakeConfig(Config& cfg, int denoise, int denoiseStep, bool doDraft, bool doNormal, bool doSlow, bool linearData);

/* OPTION_PCA for the configurations made after the call (off by default, as
   in the reference's src/Bc7Mode.h:5). */
void SetPca(bool on);


/* src/Bc7Core.h:37 */
struct Area
{
	uint16_t px[16][4];    /* pixel data, A,G,R,B */
	uint16_t mk[16][4];    /* per-channel mask, 0 or 0xFFFF */
	uint8_t idx[16];
	uint32_t count, active;
	bool opaque;
	uint8_t zero;
	uint16_t minmax[8];    /* min, max per channel */
	uint16_t bounds[8];    /* oriented endpoints per channel */
};

/* src/Bc7PcaEigen.cpp:26-146: the principal-axis error bound of an area over
   G, R, B (C = 3) or A, G, R, B (C = 4); port_pca.cpp. */
int PcaBound(const Config& cfg, const Area& area, int C);

/* src/Bc7Core.h:55 */
struct Cell
{
	V8 best0, best1, best2;
	uint64_t bestParam;
	uint32_t bestMode;

	int opaqueAlphaError;
	int errAlpha, errTotal;
	double qualityAlpha, qualityColor;

	uint64_t personalParam;
	uint32_t personalMode;

	int visibleFlags;
	int denoiseStep;
	bool opaque;

	uint16_t px[16][4];
	uint16_t mk[16][4];

	uint8_t img[16][4];   /* pixels, A,G,R,B bytes */
	uint8_t msk[16][4];   /* mask bytes, A,G,R,B */

	Area area1;
	bool lazy12[64], lazy22[64], lazy13[64], lazy23[64], lazy33[64];
	Area a12[64], a22[64], a13[64], a23[64], a33[64];
};

struct Node
{
	int err, color;
};

/* One channel's sorted candidate endpoint list (src/SnippetLevelsBuffer.h:13). */
struct Levels
{
	int minErr;
	int count;
	Node e[32];
};

void LevelsInit(Levels& L, const Config& cfg);

void MakeAreaFromCell(const Config& cfg, Area& area, const Cell& cell, int count, uint64_t indices);

Area& GetArea(const Config& cfg, Area& area, bool& lazy, const Cell& cell, uint64_t indices);

/* Error of one endpoint pair set over the active pixels of an area with a
   shared index (src/SnippetComputeOpaqueSubset2.h:7 / 3.h:7,
   src/Bc7CoreMode6.cpp:130 ComputeSubsetError4, and the ...Pair variants).
   ep: packed endpoint bytes A0 A1 G0 G1 R0 R1 B0 B1; w: per-channel weights. */
int SubsetError(const Config& cfg, const Area& area, const uint8_t ep[8], int indexBits, const int w[4], int water);

/* src/Bc7Core.cpp:746 ComputeSubsetTable<M>: per-pixel index choice with the
   SSIM tie-break.  vals[k][c] are the M interpolated levels. */
int ComputeSubsetTable(const Config& cfg, const Area& area, const int w[4], int M, const uint16_t vals[16][4], int best[16]);

void InterpolateLevels(const uint8_t ep[8], int indexBits, uint16_t vals[16][4]);

void PackEndpoints(const V8& mc, uint8_t ep[8]);

/* Per-channel candidate lists (src/SnippetLevelsBuffer.h:43,
   src/SnippetLevelsBufferHalf.h:43) and the lower-bound estimate
   (src/SnippetLevelsMinimum.h:117). */
void ChannelLevels(const Config& cfg, Levels& L, const Area& area, int offset, int weight, int water,
	int bits, int pbits, bool transparent, const uint8_t* table, bool single, int maxSize);
void ChannelLevelsHalf(const Config& cfg, Levels& L, const Area& area, int offset, int weight, int water,
	int bits, int pbits, bool transparent, const uint8_t* table, int maxSize);
int EstimateChannelLevels(const Config& cfg, const Area& area, int offset, int weight, int water,
	int bits, bool transparent, const uint8_t* table, const uint16_t* tower);

void RadixSortPartitions(Node* order, int n);

uint64_t InsertZeroBit(uint64_t value, int index);
uint64_t RemoveZeroBit(uint64_t value, int index);

void AreaReduceTable2(const Area& area, V8& mc, uint64_t& indices);
void AreaReduceTable3(const Area& area, V8& mc, uint64_t& indices);
void AreaReduceTable4(V8& mc, uint64_t& indices);

/* Block entry points (src/Bc7Core.cpp:1446, 1516). */
void DecompressBlock(const uint8_t block[16], Cell& out);
void CompressBlock(const Config& cfg, uint8_t block[16], Cell& input);

void CompareBlocks(const Config& cfg, const Cell& a, const Cell& b, int& alpha, int& total);
void CompareBlocksSSIM(const Config& cfg, const Cell& a, const Cell& b, double& alpha, double& color);

/* Mode encoders (src/Bc7CoreMode*.cpp). */
namespace mode0 { void FinalPack(const Config&, uint8_t*, Cell&); void Fast(const Config&, Cell&); void Refine(const Config&, Cell&); void Full(const Config&, Cell&); }
namespace mode1 { void FinalPack(const Config&, uint8_t*, Cell&); void Fast(const Config&, Cell&); void Refine(const Config&, Cell&); void Full(const Config&, Cell&); }
namespace mode2 { void FinalPack(const Config&, uint8_t*, Cell&); void Fast(const Config&, Cell&); void Refine(const Config&, Cell&); void Full(const Config&, Cell&); }
namespace mode3 { void FinalPack(const Config&, uint8_t*, Cell&); void Fast(const Config&, Cell&); void Refine(const Config&, Cell&); void Full(const Config&, Cell&); }
namespace mode4 { void FinalPack(const Config&, uint8_t*, Cell&); void Fast(const Config&, Cell&); void Refine(const Config&, Cell&); void Full(const Config&, Cell&); }
namespace mode5 { void FinalPack(const Config&, uint8_t*, Cell&); void Fast(const Config&, Cell&); void Refine(const Config&, Cell&); void Full(const Config&, Cell&); }
namespace mode6 { void FinalPack(const Config&, uint8_t*, Cell&); void Fast(const Config&, Cell&); void Refine(const Config&, Cell&); void Full(const Config&, Cell&); }
namespace mode6i2 { void FinalPack(const Config&, uint8_t*, Cell&); void Fast(const Config&, Cell&); void Refine(const Config&, Cell&); }
namespace mode7 { void FinalPack(const Config&, uint8_t*, Cell&); void Fast(const Config&, Cell&); void Refine(const Config&, Cell&); void Full(const Config&, Cell&); }

} // namespace nebc7_oracle
