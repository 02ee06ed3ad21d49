/*
 * BC7 block encoder for sm_103a -- device-side construction of the level
 * tables (one set per kDenoise, about 44.6 MB, kept resident).
 *
 * Entry [x][c] is the quantised distance from channel value x to the
 * nearest level interpolated between the endpoint pair c = (cH << 8) + cL:
 *   D(x, c) = q(min_k |((64 - w_k) cL + w_k cH + 32) >> 6 - x|)
 * with q(d) = d >> 1 (kDenoise = 1) or min(d, 127) (kDenoise = 0).  Reduced
 * tables keep the pairs whose endpoints are n-bit values expanded by bit
 * replication; "shared" tables mark pairs with different p-bit parity as
 * 0xFF; "half" tables hold 4-bit nibbles clamped to 15; cut tables hold the
 * squared minimum over the row prefix [0, iH | 31].  Same contents as the
 * reference's InitLevels (src/Bc7Tables.cpp:497-777); the tables with 8-bit
 * endpoints (the 2-bit byte table and the two half tables) are indexed by
 * endpoint-minus-value differences instead of by (x, c) (DiffAt, HalfAt),
 * which gives the same entries from 256 KB and 128 KB tables.
 */
#pragma once

#include "bc7_defs.cuh"

namespace nebc7 {

__global__ void KBuildFull(uint8_t* out, int levels, int denoise)
{
	/* one thread per (x, c) */
	const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (t >= uint64_t(256) * 0x10000)
		return;
	const int x = int(t >> 16);
	const int c = int(t & 0xFFFF);
	const int* w = InterpWeights(levels == 4 ? 2 : (levels == 8 ? 3 : 4));
	const int cL = c & 0xFF, cH = c >> 8;
	int best = 0x7FFF;
	for (int k = 0; k < levels; k++)
	{
		int d = Interp(cL, cH, w[k]) - x;
		d = d < 0 ? -d : d;
		best = d < best ? d : best;
	}
	out[t] = uint8_t(denoise ? (best >> denoise) : (best > 127 ? 127 : best));
}

__global__ void KReduce(const uint8_t* full, uint8_t* out, int bits, int shared)
{
	const int n = 1 << bits;
	const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (t >= uint64_t(256) * n * n)
		return;
	const int x = int(t / (n * n));
	const int r = int(t % (n * n));
	const int qH = r / n, qL = r % n;
	const int iH = qH << (8 - bits), iL = qL << (8 - bits);
	const int cH = (iH + (iH >> bits)) << 8;
	const int c = cH + iL + (iL >> bits);
	uint8_t v = full[size_t(x) * 0x10000 + c];
	if (shared && ((qH ^ qL) & 1))
		v = 0xFF;
	out[t] = v;
}

__global__ void KCut(const uint8_t* table, uint16_t* tower, int bits)
{
	const int n = 1 << bits;
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= 256 * n)
		return;
	const int x = t / n, iH = t % n;
	const uint8_t* row = table + size_t(x) * n * n + size_t(iH) * n;
	int cut = 0xFFFF;
	for (int iL = 0, hL = iH | 31; iL <= hL; iL++)
		cut = row[iL] < cut ? row[iL] : cut;
	tower[t] = uint16_t(cut * cut);
}

/* Half table by differences: byte a * 256 + bb holds the entries of
   (a, b = 2 bb) and (a, 2 bb + 1), a = cH - x + 255, b = cL - x + 255; the
   distance to level k is |(b - 255) + (((a - b) w_k + 32) >> 6)|, which is
   Interp(cL, cH, w_k) - x.  Pairs (a, b) that no (x, cL, cH) reaches are
   filled the same way and never read. */
__global__ void KBuildHalfDiff(uint8_t* out, int levels, int denoise)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= 511 * 256)
		return;
	const int a = t >> 8;
	const int* w = InterpWeights(levels == 4 ? 2 : 4);
	int res[2];
	for (int j = 0; j < 2; j++)
	{
		const int b = 2 * (t & 0xFF) + j;
		int best = 0x7FFF;
		for (int k = 0; k < levels; k++)
		{
			int d = (b - 255) + (((a - b) * w[k] + 32) >> 6);
			d = d < 0 ? -d : d;
			best = d < best ? d : best;
		}
		int q = denoise ? (best >> denoise) : (best > 127 ? 127 : best);
		res[j] = q > 15 ? 15 : q;
	}
	out[t] = uint8_t(res[0] | (res[1] << 4));
}

/* Byte table by differences (DiffAt): byte (a << 9) + b holds the entry of
   a = cH - x + 255, b = cL - x + 255, quantised like KBuildFull; column 511
   is padding. */
__global__ void KBuildByteDiff(uint8_t* out, int levels, int denoise)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= 511 * 512)
		return;
	const int a = t >> 9, b = t & 511;
	if (b == 511)
	{
		out[t] = 0;
		return;
	}
	const int* w = InterpWeights(levels == 4 ? 2 : (levels == 8 ? 3 : 4));
	int best = 0x7FFF;
	for (int k = 0; k < levels; k++)
	{
		int d = (b - 255) + (((a - b) * w[k] + 32) >> 6);
		d = d < 0 ? -d : d;
		best = d < best ? d : best;
	}
	out[t] = uint8_t(denoise ? (best >> denoise) : (best > 127 ? 127 : best));
}

} // namespace nebc7
