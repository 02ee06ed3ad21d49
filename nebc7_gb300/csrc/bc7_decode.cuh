/*
 * BC7 decode and result-reduction kernels (used by the C ABI layer only).
 */
#pragma once

#include "bc7_encode.cuh"

namespace nebc7 {

/* Decodes blocks to BGRA pixels (src/Bc7Core.cpp:1904 DecompressKernel):
   one thread per pixel. */
__global__ void KDecode(const uint8_t* blocks, uint8_t* bgra, long long stride, int blocksW, int nblocks)
{
	const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= (long long)nblocks * 16)
		return;
	const int k = int(t >> 4), i = int(t & 15);
	const uint4 b = *reinterpret_cast<const uint4*>(blocks + (long long)k * 16);
	const uint64_t lo = uint64_t(b.x) | (uint64_t(b.y) << 32);
	const uint64_t hi = uint64_t(b.z) | (uint64_t(b.w) << 32);
	uint8_t px[4];
	Ep best[3];
	int param, mode;
	DecodeBlock(lo, hi, i, px, best, param, mode);
	const int bx = k % blocksW, by = k / blocksW;
	uint8_t* p = bgra + ((long long)by * 4 + (i >> 2)) * stride + (long long)bx * 16 + (i & 3) * 4;
	*reinterpret_cast<uchar4*>(p) = make_uchar4(px[3], px[1], px[2], px[0]);
}

/* Deterministic reduction of the per-block results: a fixed-shape tree, so
   repeated runs give identical double sums. */
__global__ void KReduceResults(const BlockResult* r, int n, long long* errs, double* ssims)
{
	__shared__ long long sa[256], sc[256];
	__shared__ double qa[256], qc[256];
	const int t = threadIdx.x;
	long long a = 0, c = 0;
	double x = 0, y = 0;
	for (int i = t; i < n; i += 256)
	{
		a += r[i].errAlpha;
		c += r[i].errColor;
		x = __dadd_rn(x, r[i].ssimAlpha);
		y = __dadd_rn(y, r[i].ssimColor);
	}
	sa[t] = a;
	sc[t] = c;
	qa[t] = x;
	qc[t] = y;
	__syncthreads();
	for (int s = 128; s > 0; s >>= 1)
	{
		if (t < s)
		{
			sa[t] += sa[t + s];
			sc[t] += sc[t + s];
			qa[t] = __dadd_rn(qa[t], qa[t + s]);
			qc[t] = __dadd_rn(qc[t], qc[t + s]);
		}
		__syncthreads();
	}
	if (t == 0)
	{
		errs[0] = sa[0];
		errs[1] = sc[0];
		ssims[0] = qa[0];
		ssims[1] = qc[0];
	}
}

/* Per-texture sums of a batch: CTA t reduces the per-block results of
   table entry t (its own array, or its queue positions of r), with the
   same fixed tree as
   KReduceResults (so a texture's sums do not depend on the batch), into
   sums[tex[t].id] = { errAlpha, errColor } and ssims[...] = { alpha, color }. */
__global__ void KReduceTextures(const BlockResult* r, const TexDesc* tex, long long* errs, double* ssims)
{
	__shared__ long long sa[256], sc[256];
	__shared__ double qa[256], qc[256];
	const TexDesc& d = tex[blockIdx.x];
	const BlockResult* rr = d.results ? d.results : r + d.first;
	const int n = d.nblocks;
	const int t = threadIdx.x;
	long long a = 0, c = 0;
	double x = 0, y = 0;
	for (int i = t; i < n; i += 256)
	{
		a += rr[i].errAlpha;
		c += rr[i].errColor;
		x = __dadd_rn(x, rr[i].ssimAlpha);
		y = __dadd_rn(y, rr[i].ssimColor);
	}
	sa[t] = a;
	sc[t] = c;
	qa[t] = x;
	qc[t] = y;
	__syncthreads();
	for (int s = 128; s > 0; s >>= 1)
	{
		if (t < s)
		{
			sa[t] += sa[t + s];
			sc[t] += sc[t + s];
			qa[t] = __dadd_rn(qa[t], qa[t + s]);
			qc[t] = __dadd_rn(qc[t], qc[t + s]);
		}
		__syncthreads();
	}
	if (t == 0)
	{
		errs[2 * d.id] = sa[0];
		errs[2 * d.id + 1] = sc[0];
		ssims[2 * d.id] = qa[0];
		ssims[2 * d.id + 1] = qc[0];
	}
}

} // namespace nebc7
