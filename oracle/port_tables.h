/*
 * CPU oracle for the BC7 block encoder -- tables.  Test infrastructure only:
 * the port in this directory is the checker the CUDA encoder is compared with
 * and the CPU baseline that bench.py times; the product never links it.
 *
 * Restates reference src/Bc7Tables.cpp: BPTC interpolation weights (:7-48),
 * partition tables (:171, :242), anchor ("shrinked") tables (:313-367),
 * per-subset pixel selection lists (:377-475), the |interp - x| level tables
 * and their row-minimum "cut" tables (:478-777), and channel weights
 * (:789-844).  The partition and anchor tables are the BPTC format's own
 * (Khronos ARB_texture_compression_bptc); they are stored here as packed
 * words.
 */
#pragma once

#include <stdint.h>

namespace nebc7_oracle {

extern const int kInterp2[4];
extern const int kInterp3[8];
extern const int kInterp4[16];

/* partition p, pixel i -> subset: (kPartition2[p] >> (2*i)) & 3 */
extern const uint32_t kPartition2[64];
extern const uint32_t kPartition3[64];

extern const uint8_t kAnchor2of2[64];   /* src/Bc7Tables.cpp:313 gTableShrinked22 */
extern const uint8_t kAnchor2of3[64];   /* :325 gTableShrinked23 */
extern const uint8_t kAnchor3of3[64];   /* :337 gTableShrinked33 */

extern const int kRotationsMode4[8];    /* :847 */
extern const int kRotationsMode5[4];    /* :848 */

struct Selection
{
	uint8_t anchorLow3[64], anchorHigh3[64];          /* :349-367 */
	uint64_t sel12[64], sel22[64];                   /* :370-419 */
	uint64_t sel13[64], sel23[64], sel33[64];        /* :421-473 */
};

const Selection& GetSelection();

/* Level tables for one kDenoise value (src/Bc7Tables.cpp:478-495, 583-777). */
struct LevelTables
{
	int denoise;
	uint8_t* d2v8;   /* [256][256*256] */
	uint8_t* d2v7;   /* [256][128*128] */
	uint8_t* d2v6;   /* [256][64*64] */
	uint8_t* d2v5;   /* [256][32*32] */
	uint16_t* c2v8;  /* [256][256] */
	uint16_t* c2v6;  /* [256][64] */
	uint16_t* c2v5;  /* [256][32] */
	uint8_t* d3v7s;  /* [256][128*128] */
	uint8_t* d3v6;   /* [256][64*64] */
	uint8_t* d3v5;   /* [256][32*32] */
	uint16_t* c3v7s; /* [256][128] */
	uint16_t* c3v5;  /* [256][32] */
	uint8_t* d4h;    /* [256][256*128] nibbles */
	uint8_t* d2h;    /* [256][256*128] nibbles */
};

/* Built once per kDenoise (thread-safe); never freed. */
const LevelTables& GetLevelTables(int denoise);

} // namespace nebc7_oracle
