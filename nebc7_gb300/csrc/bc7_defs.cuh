/*
 * BC7 block encoder for sm_103a -- constants, parameters and small helpers.
 *
 * BPTC format tables (interpolation weights, partitions, anchors) are the
 * format's own (Khronos ARB_texture_compression_bptc); the reference keeps
 * the same data in src/Bc7Tables.cpp:7-48, 171-347.  They live in constant
 * memory: every lane of a warp reads the same entry (broadcast).
 */
#pragma once

#include <stdint.h>

namespace nebc7 {

/* Marks the routines that many passes call (candidate lists, estimates,
   combination searches, subset statistics): kept out of line so the kernel
   holds one copy of each and its working set fits the instruction cache. */
#ifndef NEBC7_SHARED
#define NEBC7_SHARED __noinline__
#endif

/* Marks the pass-level routines of the refinement and full searches (one
   refinement, one full search of a mode, a subset search, an estimate
   pass).  The outlined kernels define it __noinline__: with the passes
   inlined into the kernel body its code outgrows the instruction cache, and
   warps that sit in different passes stall on instruction fetch.  Empty
   by default (the compiler decides). */
#ifndef NEBC7_PASS
#define NEBC7_PASS
#endif

/* Marks the passes a block runs once (the fast passes, the final pack).  The
   draft-only translation units define it __noinline__; in the kernels with
   the searches, out-of-line copies raise the register count (232 -> 247). */
#ifndef NEBC7_ONCE
#define NEBC7_ONCE
#endif


static __constant__ int c_interp2[4] = { 0, 21, 43, 64 };
static __constant__ int c_interp3[8] = { 0, 9, 18, 27, 37, 46, 55, 64 };
static __constant__ int c_interp4[16] = { 0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64 };

/* subset of pixel i in partition p: (c_part[p] >> 2i) & 3 */
static __constant__ uint32_t c_part2[64] = {
	0x50505050u, 0x40404040u, 0x54545454u, 0x54505040u, 0x50404000u, 0x55545450u, 0x55545040u, 0x54504000u,
	0x50400000u, 0x55555450u, 0x55544000u, 0x54400000u, 0x55555440u, 0x55550000u, 0x55555500u, 0x55000000u,
	0x55150100u, 0x00004054u, 0x15010000u, 0x00405054u, 0x00004050u, 0x15050100u, 0x05010000u, 0x40505054u,
	0x00404050u, 0x05010100u, 0x14141414u, 0x05141450u, 0x01155440u, 0x00555500u, 0x15014054u, 0x05414150u,
	0x44444444u, 0x55005500u, 0x11441144u, 0x05055050u, 0x05500550u, 0x11114444u, 0x41144114u, 0x44111144u,
	0x15055054u, 0x01055040u, 0x05041050u, 0x05455150u, 0x14414114u, 0x50050550u, 0x41411414u, 0x00141400u,
	0x00041504u, 0x00105410u, 0x10541000u, 0x04150400u, 0x50410514u, 0x41051450u, 0x05415014u, 0x14054150u,
	0x41050514u, 0x41505014u, 0x40011554u, 0x54150140u, 0x50505500u, 0x00555050u, 0x15151010u, 0x54540404u,
};
static __constant__ uint32_t c_part3[64] = {
	0xAA685050u, 0x6A5A5040u, 0x5A5A4200u, 0x5450A0A8u, 0xA5A50000u, 0xA0A05050u, 0x5555A0A0u, 0x5A5A5050u,
	0xAA550000u, 0xAA555500u, 0xAAAA5500u, 0x90909090u, 0x94949494u, 0xA4A4A4A4u, 0xA9A59450u, 0x2A0A4250u,
	0xA5945040u, 0x0A425054u, 0xA5A5A500u, 0x55A0A0A0u, 0xA8A85454u, 0x6A6A4040u, 0xA4A45000u, 0x1A1A0500u,
	0x0050A4A4u, 0xAAA59090u, 0x14696914u, 0x69691400u, 0xA08585A0u, 0xAA821414u, 0x50A4A450u, 0x6A5A0200u,
	0xA9A58000u, 0x5090A0A8u, 0xA8A09050u, 0x24242424u, 0x00AA5500u, 0x24924924u, 0x24499224u, 0x50A50A50u,
	0x500AA550u, 0xAAAA4444u, 0x66660000u, 0xA5A0A5A0u, 0x50A050A0u, 0x69286928u, 0x44AAAA44u, 0x66666600u,
	0xAA444444u, 0x54A854A8u, 0x95809580u, 0x96969600u, 0xA85454A8u, 0x80959580u, 0xAA141414u, 0x96960000u,
	0xAAAA1414u, 0xA05050A0u, 0xA0A5A5A0u, 0x96000000u, 0x40804080u, 0xA9A8A9A8u, 0xAAAAAA44u, 0x2A4A5254u,
};
static __constant__ uint8_t c_anchor22[64] = {
	15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 2, 8, 2, 2, 8, 8, 15, 2, 8, 2, 2, 8, 8, 2, 2,
	15, 15, 6, 8, 2, 8, 15, 15, 2, 8, 2, 2, 2, 15, 15, 6, 6, 2, 6, 8, 15, 15, 2, 2, 15, 15, 15, 15, 15, 2, 2, 15,
};
static __constant__ uint8_t c_anchor23[64] = {
	3, 3, 15, 15, 8, 3, 15, 15, 8, 8, 6, 6, 6, 5, 3, 3, 3, 3, 8, 15, 3, 3, 6, 10, 5, 8, 8, 6, 8, 5, 15, 15,
	8, 15, 3, 5, 6, 10, 8, 15, 15, 3, 15, 5, 15, 15, 15, 15, 3, 15, 5, 5, 5, 8, 5, 10, 5, 10, 8, 13, 15, 12, 3, 3,
};
static __constant__ uint8_t c_anchor33[64] = {
	15, 8, 8, 3, 15, 15, 3, 8, 15, 15, 15, 15, 15, 15, 15, 8, 15, 8, 15, 3, 15, 8, 15, 8, 3, 15, 6, 10, 15, 15, 10, 8,
	15, 3, 15, 10, 10, 8, 9, 10, 6, 15, 8, 15, 3, 6, 6, 8, 15, 3, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 3, 15, 15, 8,
};
/* rotation visiting orders, mode 4 (rotation | idxMode << 2) and mode 5 */
static __constant__ int c_rot4[8] = { 4, 0, 6, 2, 5, 1, 7, 3 };
static __constant__ int c_rot5[4] = { 0, 2, 1, 3 };

/* Level tables for one kDenoise value, resident in device memory (layouts
   and contents as described in the table builder). */
struct LevelTables
{
	const uint8_t* d2v8;   /* [511][512] bytes, by differences (DiffAt) */
	const uint8_t* d2v7;   /* [256][128*128] */
	const uint8_t* d2v6;   /* [256][64*64]   */
	const uint8_t* d2v5;   /* [256][32*32]   */
	const uint16_t* c2v8;  /* [256][256]     */
	const uint16_t* c2v6;  /* [256][64]      */
	const uint16_t* c2v5;  /* [256][32]      */
	const uint8_t* d3v7s;  /* [256][128*128] */
	const uint8_t* d3v6;   /* [256][64*64]   */
	const uint8_t* d3v5;   /* [256][32*32]   */
	const uint16_t* c3v7s; /* [256][128]     */
	const uint16_t* c3v5;  /* [256][32]      */
	const uint8_t* d4h;    /* [511][256] nibbles, by differences (HalfAt) */
	const uint8_t* d2h;    /* [511][256] nibbles, by differences (HalfAt) */
	const uint8_t* d3v8;   /* [511][512] bytes of 3-bit indices, by differences (DiffAt) */
};

/* Per-launch encoder settings: the reference's InitTables flags
   (src/Bc7Core.cpp:1877) and channel weights (src/Bc7Tables.cpp:789). */
struct Params
{
	int denoiseStep;            /* kDenoiseStep */
	int wA, wG, wR, wB;
	int wColor, wColorAlpha;
	int doDraft, doNormal, doSlow;
	int pca;                    /* OPTION_PCA bounds in the full searches (off by default) */
};

template<int kD>
__device__ __forceinline__ int Q(int d)
{
	d = d < 0 ? -d : d;
	if (kD)
		return d >> kD;
	return d > 127 ? 127 : d;
}

template<int kD>
__device__ __forceinline__ int MaxColorError()
{
	return 16 * (255 >> kD) * (255 >> kD) * 1000 + 1;
}

__device__ __forceinline__ int Interp(int e0, int e1, int w)
{
	return (e0 * (64 - w) + e1 * w + 32) >> 6;
}

/* Entry (x, cL, cH) of a nibble table: the quantised distance from x to the
   nearest level of the 8-bit endpoint pair, clamped to 15.  The levels are
   cL + (((cH - cL) w + 32) >> 6), so the entry depends on cH - x and cL - x
   only: one 511 x 511 table serves every x (row cH - x + 255, nibble
   cL - x + 255), 128 KB instead of 256 rows of 32 KB, and the rows a block
   touches stay in L1. */
__device__ __forceinline__ int HalfAt(const uint8_t* table, int x, int cL, int cH)
{
	const int a = cH - x + 255, b = cL - x + 255;
	return (table[a * 256 + (b >> 1)] >> ((b & 1) << 2)) & 0xF;
}

/* Entry (x, cL, cH) of the 8-bit-endpoint byte table of 2-bit indices, the
   same function of cH - x and cL - x as HalfAt's, unclamped: rows of 512
   bytes (511 used) by cH - x + 255, columns by cL - x + 255, 256 KB for every
   x instead of 256 rows of 64 KB. */
__device__ __forceinline__ int DiffAt(const uint8_t* table, int x, int cL, int cH)
{
	return table[((cH - x + 255) << 9) + (cL - x + 255)];
}

__device__ __forceinline__ const int* InterpWeights(int bits)
{
	return bits == 2 ? c_interp2 : (bits == 3 ? c_interp3 : c_interp4);
}

__device__ __forceinline__ uint64_t InsertZeroBit(uint64_t value, int index)
{
	uint64_t high = (~uint64_t(0) << index) & value;
	return (value ^ high) + (high << 1);
}

/* Channel in the alpha-index slot of a mode 4/5 rotation: A, R, G, B. */
__device__ __forceinline__ int RotChannel(int rotation)
{
	const int r = rotation & 3;
	return r == 0 ? 0 : (r == 1 ? 2 : (r == 2 ? 1 : 3));
}

constexpr unsigned kFull = 0xFFFFFFFFu;

} // namespace nebc7
