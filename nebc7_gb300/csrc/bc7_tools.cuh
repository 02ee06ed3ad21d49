/*
 * BC7 block encoder for sm_103a -- the steps around the encode that the
 * reference's command-line driver runs on the host: texture padding and the
 * alpha outline mask (src/Bc7Compress.cpp:20-105, :397-426, :470-477), the
 * glitch map of /bad (src/Worker.cpp:309-451) and the partition map of /map
 * (src/Bc7Compress.cpp:131-265).  All run on device buffers.
 */
#pragma once

#include "bc7_defs.cuh"
#include "bc7_encode.cuh"

namespace nebc7 {

/* Edge replication of a w x h BGRA image to the padded pw x ph texture:
   columns past w repeat column w - 1, rows past h repeat row h - 1. */
__global__ void KPadTexture(const uint8_t* src, long long srcStride, int w, int h, uint8_t* dst, long long dstStride, int pw,
	int ph)
{
	const int x = blockIdx.x * blockDim.x + threadIdx.x;
	const int y = blockIdx.y;
	if (x >= pw || y >= ph)
		return;
	const int sx = x < w ? x : w - 1;
	const int sy = y < h ? y : h - 1;
	*reinterpret_cast<uint32_t*>(dst + y * dstStride + x * 4) =
		*reinterpret_cast<const uint32_t*>(src + sy * srcStride + sx * 4);
}

/* Alpha mask with an outline: bytes A, G, R, B of a pixel are 0xFF, and G,
   R, B are 0xFF only if some pixel of the (2 radius + 1)^2 window around it
   (clipped to the texture) has non-zero alpha.  radius < 0: all 0xFF. */
__global__ void KOutlineMask(const uint8_t* tex, long long stride, int pw, int ph, int radius, uint8_t* mask)
{
	const int x = blockIdx.x * blockDim.x + threadIdx.x;
	const int y = blockIdx.y;
	if (x >= pw || y >= ph)
		return;
	uint32_t m = 0xFFFFFFFFu;
	if (radius >= 0)
	{
		bool any = false;
		for (int yy = max(0, y - radius); yy <= min(ph - 1, y + radius) && !any; yy++)
			for (int xx = max(0, x - radius); xx <= min(pw - 1, x + radius); xx++)
				if (tex[yy * stride + xx * 4 + 3])
				{
					any = true;
					break;
				}
		m = any ? 0xFFFFFFFFu : 0x000000FFu;
	}
	*reinterpret_cast<uint32_t*>(mask + y * stride + x * 4) = m;
}

/* Glitch map: a block whose decoded pixels differ from the source by at
   least the threshold in some masked channel (A 16, G 12, R 16, B 20;
   16 each with linear weights) keeps its source pixels, any other block is
   cleared.  One thread per pixel; the block's verdict by warp vote over its
   16 pixels (a warp holds two blocks side by side). */
__global__ void KBadBlocks(const uint8_t* src, const uint8_t* dec, const uint8_t* mask, long long stride, int w, int h, int linear,
	uint8_t* out)
{
	const int bx = blockIdx.x * 2 + (threadIdx.x >> 4);
	const int by = blockIdx.y;
	const int i = threadIdx.x & 15;
	const bool in = bx * 4 < w && by * 4 < h;
	const long long off = (long long)(by * 4 + (i >> 2)) * stride + (bx * 4 + (i & 3)) * 4;
	bool bad = false;
	uint32_t s = 0;
	if (in)
	{
		s = *reinterpret_cast<const uint32_t*>(src + off);
		const uint32_t d = *reinterpret_cast<const uint32_t*>(dec + off);
		const uint32_t m = mask ? *reinterpret_cast<const uint32_t*>(mask + off) : 0xFFFFFFFFu;
		/* BGRA bytes; mask bytes are A, G, R, B */
		const int thrB = linear ? 16 : 20, thrG = linear ? 16 : 12, thrR = 16, thrA = 16;
		const int chB = abs(int(s & 0xFF) - int(d & 0xFF)) & int(m >> 24);
		const int chG = abs(int((s >> 8) & 0xFF) - int((d >> 8) & 0xFF)) & int((m >> 8) & 0xFF);
		const int chR = abs(int((s >> 16) & 0xFF) - int((d >> 16) & 0xFF)) & int((m >> 16) & 0xFF);
		const int chA = abs(int(s >> 24) - int(d >> 24)) & int(m & 0xFF);
		bad = chB >= thrB || chG >= thrG || chR >= thrR || chA >= thrA;
	}
	const unsigned votes = __ballot_sync(0xFFFFFFFFu, bad);
	const bool blockBad = (votes >> (threadIdx.x & 16)) & 0xFFFF;
	if (in)
		*reinterpret_cast<uint32_t*>(out + off) = blockBad ? s : 0u;
}

/* Partition map: every block keeps its mode and partition (or rotation)
   bits and gets fixed endpoints, so that its decoded pixels show the
   subsets as flat colours: one channel ramp per subset, a grey for mode 6
   (two greys: whether its indices have a 2-bit pattern), mode 4 / 5 tinted
   by their alpha.  The bit values are the map's definition
   (src/Bc7Compress.cpp:131-265).  One thread per block. */
__global__ void KPartitionMap(const uint8_t* blocks, uint8_t* out, int n)
{
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= n)
		return;
	const uint4 b = reinterpret_cast<const uint4*>(blocks)[k];
	uint64_t d0 = uint64_t(b.x) | (uint64_t(b.y) << 32);
	uint64_t d1 = uint64_t(b.z) | (uint64_t(b.w) << 32);
	const int mode = (d0 & 0xFF) ? __ffs(int(d0 & 0xFF)) - 1 : 8;
	switch (mode)
	{
	case 0:   /* 4-bit partition */
		d0 = (d0 & 0x1F) | (0xFull << 29) | (0xFull << 13);
		d1 = 0xFull << 5;
		break;
	case 1:   /* 6-bit partition */
		d0 = (d0 & 0xFF) | (0x3Full << 32) | (0x3Full << 20);
		d1 = 0;
		break;
	case 2:
		d0 = (d0 & 0x1FF) | (0x1Full << 39) | (0x1Full << 19);
		d1 = 0x1Full << 25;
		break;
	case 3:
		d0 = (d0 & 0x3FF) | (0x7Full << 38) | (0x7Full << 24);
		d1 = 0;
		break;
	case 4:   /* mode bits only */
		d0 = (d0 & 0x1F) | (0x1Full << 18) | (0x1Full << 8) | (0x3Full << 38);
		d1 = 0;
		break;
	case 5:
		d0 = (d0 & 0x3F) | (0x7Full << 22) | (0x7Full << 8) | (0xFFull << 50);
		d1 = 0;
		break;
	case 6:
		if (d0 == 0x40 && d1 == 0)
			break;   /* the empty block stays */
		{
			/* indices with the anchor's missing bit re-inserted as 0 */
			const uint64_t idx = (d1 & ~0xFull) + ((d1 & 0xFull) >> 1);
			const uint64_t c = (((idx >> 2) ^ idx) & 0x3333333333333333ull) ? 0x50 : 0x30;
			d0 = (d0 & 0x7F) | (c << 21) | (c << 7) | (c << 35) | (0x7Full << 49);
			d1 = 0;
		}
		break;
	case 7:
		d0 = (d0 & 0x3FFF) | (0x1Full << 34) | (0x1Full << 24);
		d1 = (0x1Full << 10) | (0x1Full << 20);
		break;
	default:  /* no mode: unchanged */
		break;
	}
	reinterpret_cast<uint4*>(out)[k] = make_uint4(unsigned(d0), unsigned(d0 >> 32), unsigned(d1), unsigned(d1 >> 32));
}

/* Hot-first block order of one texture.  The blocks of a texture are
   independent and each writes its own slots, so the order in which a launch
   takes them changes nothing in its output; taking the blocks with the
   widest pixel ranges (the long searches) first leaves short ones for the
   end of the launch.  KBlockBuckets: bucket 255 - min(255, range / 4) per
   block, range = sum over B, G, R, A of max - min over its 16 pixels, and a
   histogram of the buckets (zero before the launch). */
__global__ void KBlockBuckets(const uint8_t* bgra, long long stride, int blocksW, int nblocks, uint8_t* bucket, int* hist)
{
	__shared__ int h[256];
	for (int i = threadIdx.x; i < 256; i += blockDim.x)
		h[i] = 0;
	__syncthreads();
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k < nblocks)
	{
		const int bx = k % blocksW, by = k / blocksW;
		const uint8_t* p = bgra + (long long)by * 4 * stride + (long long)bx * 16;
		unsigned lo = 0xFFFFFFFFu, hi = 0;
		for (int r = 0; r < 4; r++)
			for (int x = 0; x < 4; x++)
			{
				const unsigned v = *reinterpret_cast<const uint32_t*>(p + r * stride + x * 4);
				lo = __vminu4(lo, v);
				hi = __vmaxu4(hi, v);
			}
		const unsigned d = __vsubus4(hi, lo);
		const int range = int(d & 0xFF) + int((d >> 8) & 0xFF) + int((d >> 16) & 0xFF) + int(d >> 24);
		const int b = 255 - min(255, range >> 2);
		bucket[k] = uint8_t(b);
		atomicAdd(&h[b], 1);
	}
	__syncthreads();
	for (int i = threadIdx.x; i < 256; i += blockDim.x)
		if (h[i])
			atomicAdd(&hist[i], h[i]);
}

/* Expected-cost class of a texture's preset (the measured cost ratios
   draft 1, default 11, precise 400, /slow 480, /data 7200 of a block). */
__device__ __forceinline__ int CostClass(const TexDesc& d)
{
	if (!d.P.doNormal || d.P.doDraft == 2)
		return 0;
	if (d.P.wA == 1)
		return 3;
	if (d.P.doSlow || d.denoise == 0 || d.P.denoiseStep == 0)
		return 2;
	return 1;
}

/* KBlockBuckets over the queue of a launch of several textures: bucket
   255 - (64 * cost class + min(63, range / 16)) per queue position, so that
   the counting sort deals the most expensive preset's widest blocks first. */
__global__ void KJobBuckets(const TexDesc* tex, int ntex, int total, uint8_t* bucket, int* hist)
{
	__shared__ int h[256];
	for (int i = threadIdx.x; i < 256; i += blockDim.x)
		h[i] = 0;
	__syncthreads();
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k < total)
	{
		int t = 0, hi = ntex - 1;
		while (t < hi)
		{
			const int mid = (t + hi + 1) >> 1;
			if (tex[mid].first <= k)
				t = mid;
			else
				hi = mid - 1;
		}
		const TexDesc& d = tex[t];
		const int local = k - d.first;
		const int bx = local % d.blocksW, by = local / d.blocksW;
		const uint8_t* p = d.bgra + (long long)by * 4 * d.stride + (long long)bx * 16;
		unsigned lo = 0xFFFFFFFFu, hv = 0;
		for (int r = 0; r < 4; r++)
			for (int x = 0; x < 4; x++)
			{
				const unsigned v = *reinterpret_cast<const uint32_t*>(p + r * d.stride + x * 4);
				lo = __vminu4(lo, v);
				hv = __vmaxu4(hv, v);
			}
		const unsigned dd = __vsubus4(hv, lo);
		const int range = int(dd & 0xFF) + int((dd >> 8) & 0xFF) + int((dd >> 16) & 0xFF) + int(dd >> 24);
		const int b = 255 - (64 * CostClass(d) + min(63, range >> 4));
		bucket[k] = uint8_t(b);
		atomicAdd(&h[b], 1);
	}
	__syncthreads();
	for (int i = threadIdx.x; i < 256; i += blockDim.x)
		if (h[i])
			atomicAdd(&hist[i], h[i]);
}

/* Counting-sort scatter: order[] lists the blocks bucket by bucket (any
   order inside a bucket); cursor[] is zero before the launch.  256 threads
   per CTA, every thread of a warp reaching the warp-wide steps. */
__global__ void KBlockOrder(const uint8_t* bucket, int nblocks, const int* hist, int* cursor, int* order)
{
	__shared__ int base[256];
	if (threadIdx.x < 32)
	{
		/* exclusive scan of the 256 counts: 8 per lane, then across lanes */
		const int lane = threadIdx.x;
		int c[8], run = 0;
		for (int j = 0; j < 8; j++)
		{
			c[j] = run;
			run += hist[lane * 8 + j];
		}
		int incl = run;
		for (int o = 1; o < 32; o <<= 1)
		{
			const int v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
			if (lane >= o)
				incl += v;
		}
		const int excl = incl - run;
		for (int j = 0; j < 8; j++)
			base[lane * 8 + j] = excl + c[j];
	}
	__syncthreads();
	/* one atomic per distinct bucket of a warp (most blocks of a texture
	   share a few buckets) */
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	const int lane = threadIdx.x & 31;
	const int b = k < nblocks ? int(bucket[k]) : 256 + lane;
	const unsigned peers = __match_any_sync(0xFFFFFFFFu, b);
	const int leader = __ffs(peers) - 1;
	int pos = 0;
	if (lane == leader && b < 256)
		pos = atomicAdd(&cursor[b], __popc(peers));
	pos = __shfl_sync(0xFFFFFFFFu, pos, leader);
	if (k < nblocks)
		order[base[b] + pos + __popc(peers & ((1u << lane) - 1))] = k;
}

} // namespace nebc7
