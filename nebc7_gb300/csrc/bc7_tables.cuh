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
 * reference's InitLevels (src/Bc7Tables.cpp:497-777).
 */
#pragma once

#include "bc7_defs.cuh"

namespace nebc7 {

__global__ void KBuildFull(uint8_t* out, int levels, int denoise, int clampNibble)
{
	/* one thread per (x, c); nibble tables: one thread per (x, even c) */
	const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	const int per = clampNibble ? 0x8000 : 0x10000;
	if (t >= uint64_t(256) * per)
		return;
	const int x = int(t / per);
	const int r = int(t % per);
	const int* w = InterpWeights(levels == 4 ? 2 : (levels == 8 ? 3 : 4));
	int res[2];
	const int nc = clampNibble ? 2 : 1;
	for (int j = 0; j < nc; j++)
	{
		const int c = clampNibble ? 2 * r + j : r;
		const int cL = c & 0xFF, cH = c >> 8;
		int best = 0x7FFF;
		for (int k = 0; k < levels; k++)
		{
			int d = Interp(cL, cH, w[k]) - x;
			d = d < 0 ? -d : d;
			best = d < best ? d : best;
		}
		int q = denoise ? (best >> denoise) : (best > 127 ? 127 : best);
		if (clampNibble && q > 15)
			q = 15;
		res[j] = q;
	}
	if (clampNibble)
		out[t] = uint8_t(res[0] | (res[1] << 4));
	else
		out[t] = uint8_t(res[0]);
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

__global__ void KHalfFrom2(const uint8_t* d2v8, uint8_t* d2h)
{
	const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (t >= uint64_t(256) * 0x8000)
		return;
	const int x = int(t / 0x8000), r = int(t % 0x8000);
	int v0 = d2v8[size_t(x) * 0x10000 + 2 * r];
	int v1 = d2v8[size_t(x) * 0x10000 + 2 * r + 1];
	v0 = v0 > 15 ? 15 : v0;
	v1 = v1 > 15 ? 15 : v1;
	d2h[t] = uint8_t(v0 | (v1 << 4));
}

} // namespace nebc7
