/*
 * nebc7_gb300 -- host side of the C ABI declared in include/nebc7_gb300.h.
 *
 * Owns the per-device resident level tables (built on the device the first
 * time a preset's kDenoise is used), launches the persistent encode kernel
 * with stream-ordered scratch (work counter, per-block results), and adapts
 * the reference's IBc7Core / ProcessTexture interfaces onto it.
 */
#include "bc7_tables.cuh"
#include "bc7_decode.cuh"
#include "bc7_staged.cuh"
#include "bc7_tools.cuh"

#include "../../include/nebc7_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string.h>
#include <thread>
#include <unordered_map>
#include <vector>

using namespace nebc7;

namespace {

constexpr int kMaxDevices = 16;

struct DeviceTables
{
	bool built = false;
	LevelTables t{};
	void* mem[15] = {};
};

std::mutex gMutex;
DeviceTables gTables[kMaxDevices][2];
int gLastError = NEBC7_OK;

/* InitTables state of the IBc7Core adapter (src/Bc7Core.cpp:20-22, 1877) */
nebc7_settings gCore = { 1, 9, 1, 1, 0, 0 };

int SetError(int e)
{
	gLastError = e;
	return e;
}

#define CK(x)                                \
	do                                       \
	{                                        \
		if ((x) != cudaSuccess)              \
			return SetError(NEBC7_ECUDA);    \
	} while (0)

/* Bytes of each resident level table, in LevelTables order. */
constexpr int kNumLevelTables = 15;
constexpr size_t kLevelTableBytes[kNumLevelTables] = {
	size_t(511) * 512, size_t(256) * 16384, size_t(256) * 4096, size_t(256) * 1024,
	size_t(256) * 256 * 2, size_t(256) * 64 * 2, size_t(256) * 32 * 2,
	size_t(256) * 16384, size_t(256) * 4096, size_t(256) * 1024,
	size_t(256) * 128 * 2, size_t(256) * 32 * 2,
	size_t(511) * 256, size_t(511) * 256,
	size_t(511) * 512,
};

int BuildTables(int dev, int denoise, const LevelTables** out)
{
	std::lock_guard<std::mutex> lock(gMutex);
	if (dev < 0 || dev >= kMaxDevices)
		return SetError(NEBC7_EINVAL);
	DeviceTables& D = gTables[dev][denoise];
	if (!D.built)
	{
		const size_t* sizes = kLevelTableBytes;
		/* per-x full tables, only to build the reduced and cut tables from */
		uint8_t* d3v8 = nullptr;
		uint8_t* d2v8 = nullptr;
		/* a failed build leaves nothing allocated, so a later call starts over */
		auto release = [&]() {
			for (void*& m : D.mem)
			{
				cudaFree(m);
				m = nullptr;
			}
			cudaFree(d3v8);
			cudaFree(d2v8);
		};
		for (int i = 0; i < kNumLevelTables; i++)
		{
			if (cudaMalloc(&D.mem[i], sizes[i]) != cudaSuccess)
			{
				release();
				return SetError(NEBC7_ENOMEM);
			}
		}
		if (cudaMalloc(&d3v8, size_t(256) * 65536) != cudaSuccess ||
			cudaMalloc(&d2v8, size_t(256) * 65536) != cudaSuccess)
		{
			release();
			return SetError(NEBC7_ENOMEM);
		}
		const int tb = 256;
		auto grid = [&](uint64_t n) { return unsigned((n + tb - 1) / tb); };
		/* 3-bit index tables (reference src/Bc7Tables.cpp:587-641) */
		KBuildFull<<<grid(uint64_t(256) * 65536), tb>>>(d3v8, 8, denoise);
		KReduce<<<grid(uint64_t(256) * 16384), tb>>>(d3v8, (uint8_t*)D.mem[7], 7, 1);
		KReduce<<<grid(uint64_t(256) * 4096), tb>>>(d3v8, (uint8_t*)D.mem[8], 6, 0);
		KReduce<<<grid(uint64_t(256) * 1024), tb>>>(d3v8, (uint8_t*)D.mem[9], 5, 0);
		KCut<<<grid(256 * 128), tb>>>((uint8_t*)D.mem[7], (uint16_t*)D.mem[10], 7);
		KCut<<<grid(256 * 32), tb>>>((uint8_t*)D.mem[9], (uint16_t*)D.mem[11], 5);
		/* 2-bit index tables (:643-692) */
		KBuildFull<<<grid(uint64_t(256) * 65536), tb>>>(d2v8, 4, denoise);
		KReduce<<<grid(uint64_t(256) * 16384), tb>>>(d2v8, (uint8_t*)D.mem[1], 7, 0);
		KReduce<<<grid(uint64_t(256) * 4096), tb>>>(d2v8, (uint8_t*)D.mem[2], 6, 0);
		KReduce<<<grid(uint64_t(256) * 1024), tb>>>(d2v8, (uint8_t*)D.mem[3], 5, 0);
		KCut<<<grid(256 * 256), tb>>>(d2v8, (uint16_t*)D.mem[4], 8);
		KCut<<<grid(256 * 64), tb>>>((uint8_t*)D.mem[2], (uint16_t*)D.mem[5], 6);
		KCut<<<grid(256 * 32), tb>>>((uint8_t*)D.mem[3], (uint16_t*)D.mem[6], 5);
		/* 4-bit and 2-of-4-bit nibble tables (:694-776) */
		KBuildHalfDiff<<<grid(511 * 256), tb>>>((uint8_t*)D.mem[12], 16, denoise);
		KBuildHalfDiff<<<grid(511 * 256), tb>>>((uint8_t*)D.mem[13], 4, denoise);
		KBuildByteDiff<<<grid(511 * 512), tb>>>((uint8_t*)D.mem[0], 4, denoise);
		KBuildByteDiff<<<grid(511 * 512), tb>>>((uint8_t*)D.mem[14], 8, denoise);
		const cudaError_t e = cudaDeviceSynchronize();
		cudaFree(d3v8);
		cudaFree(d2v8);
		d3v8 = d2v8 = nullptr;
		if (e != cudaSuccess)
		{
			release();
			return SetError(NEBC7_ECUDA);
		}
		LevelTables& t = D.t;
		t.d2v8 = (const uint8_t*)D.mem[0];
		t.d2v7 = (const uint8_t*)D.mem[1];
		t.d2v6 = (const uint8_t*)D.mem[2];
		t.d2v5 = (const uint8_t*)D.mem[3];
		t.c2v8 = (const uint16_t*)D.mem[4];
		t.c2v6 = (const uint16_t*)D.mem[5];
		t.c2v5 = (const uint16_t*)D.mem[6];
		t.d3v7s = (const uint8_t*)D.mem[7];
		t.d3v6 = (const uint8_t*)D.mem[8];
		t.d3v5 = (const uint8_t*)D.mem[9];
		t.c3v7s = (const uint16_t*)D.mem[10];
		t.c3v5 = (const uint16_t*)D.mem[11];
		t.d4h = (const uint8_t*)D.mem[12];
		t.d2h = (const uint8_t*)D.mem[13];
		t.d3v8 = (const uint8_t*)D.mem[14];
		D.built = true;
	}
	*out = &D.t;
	return NEBC7_OK;
}

/* OPTION_PCA for the launches and plans made after nebc7_set_pca. */
std::atomic<int> gPca{ 0 };

Params MakeParams(const nebc7_settings& s)
{
	Params p;
	p.pca = gPca.load();
	p.denoiseStep = s.denoiseStep;
	if (s.linearData)
	{
		p.wA = p.wG = p.wR = p.wB = 1;
	}
	else
	{
		p.wA = 1000;
		p.wG = 715;
		p.wR = 213;
		p.wB = 72;
	}
	p.wColor = p.wG + p.wR + p.wB;
	p.wColorAlpha = p.wColor + p.wA;
	p.doDraft = s.doDraft;
	p.doNormal = s.doNormal;
	p.doSlow = s.doSlow;
	return p;
}

int ValidateSettings(const nebc7_settings* s)
{
	if (!s || (s->denoise != 0 && s->denoise != 1) || s->denoiseStep < 0 || s->denoiseStep > 4096 || s->doDraft < 0 ||
		s->doDraft > 2)
		return NEBC7_EINVAL;
	if ((s->doNormal || s->doSlow) && !kHasNormalPasses)
		return NEBC7_EUNSUPPORTED;
	return NEBC7_OK;
}

/* The encode instantiations: denoise shift x passes x code shape.  The
   outlined ones also have a staged form (bc7_staged.cuh: one kernel per
   pass), used where the launch has room for its per-block records; the
   single kernel serves the allocation-free entry and the request loop. */
struct EncodeVariant
{
	cudaError_t (*launch)(int, cudaStream_t, const Job&, const LevelTables&, const LevelTables&);
	cudaError_t (*occupancy)(int*);
	cudaError_t (*staged)(int, cudaStream_t, const Job&, const Stages&, const LevelTables&, const LevelTables&);
	cudaError_t (*stagedOccupancy)(int*);
};

constexpr int kNumVariants = 6;
constexpr int kVariantMixed = 5;   /* batches: kDenoise per texture */
const EncodeVariant kVariants[kNumVariants] = {
	{ LaunchEncodeKernel<0, false, kShapeCompact>, EncodeKernelOccupancy<0, false, kShapeCompact>, nullptr, nullptr },
	{ LaunchEncodeKernel<0, true, kShapeOutlined>, EncodeKernelOccupancy<0, true, kShapeOutlined>,
	  LaunchStagedEncode<0>, StagedEncodeOccupancy<0> },
	{ LaunchEncodeKernel<1, false, kShapeCompact>, EncodeKernelOccupancy<1, false, kShapeCompact>, nullptr, nullptr },
	{ LaunchEncodeKernel<1, true, kShapeCompact>, EncodeKernelOccupancy<1, true, kShapeCompact>, nullptr, nullptr },
	{ LaunchEncodeKernel<1, true, kShapeOutlined>, EncodeKernelOccupancy<1, true, kShapeOutlined>,
	  LaunchStagedEncode<1>, StagedEncodeOccupancy<1> },
	{ LaunchEncodeKernel<kAnyDenoise, true, kShapeOutlined>, EncodeKernelOccupancy<kAnyDenoise, true, kShapeOutlined>,
	  LaunchStagedEncode<kAnyDenoise>, StagedEncodeOccupancy<kAnyDenoise> },
};

bool SlotStaged(int slot)
{
	return kVariants[slot].staged != nullptr;
}

/* Picks the instantiation: the compact shape for the stepped default preset
   (kDenoise 1, refinement without /slow or /data), the outlined one where
   the full searches dominate (measured on the 1024x1024 and 2048x2048
   workloads). */
int VariantSlot(const nebc7_settings& s)
{
	if (!s.doNormal || s.doDraft == 2)
		return s.denoise ? 2 : 0;
	if (!s.denoise)
		return 1;
	return (s.doSlow || s.linearData) ? 4 : 3;
}

/* Launch shape of one encode instantiation on one device, looked up once
   (with the device current): this also raises the kernel's dynamic
   shared-memory limit, so it runs before the first launch on the device. */
struct LaunchShape
{
	int sms = 0;
	int perSm[kNumVariants] = {};
};

std::mutex gShapeMutex;
LaunchShape gShapes[kMaxDevices];

/* Grid of a persistent launch of `slot` over nblocks blocks: one CTA per
   kWarpsPerCta blocks up to the resident CTAs of every SM, or up to
   ctasPerSm per SM when that is given (> 0) and smaller. */
int GridForSlotCap(int nblocks, int slot, int ctasPerSm);

int GridForSlot(int nblocks, int slot)
{
	return GridForSlotCap(nblocks, slot, 0);
}

int GridForSlotCap(int nblocks, int slot, int ctasPerSm)
{
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
		return 0;
	int sms, perSm;
	{
		std::lock_guard<std::mutex> lock(gShapeMutex);
		LaunchShape& L = gShapes[dev];
		if (!L.sms)
		{
			cudaDeviceGetAttribute(&L.sms, cudaDevAttrMultiProcessorCount, dev);
			if (L.sms <= 0)
				L.sms = 1;
		}
		if (!L.perSm[slot])
		{
			int n = 0;
			if (kVariants[slot].occupancy(&n) != cudaSuccess)
				return 0;
			if (kVariants[slot].stagedOccupancy)
			{
				/* prepares the stage kernels too; the grid fits both forms */
				int m = 0;
				if (kVariants[slot].stagedOccupancy(&m) != cudaSuccess)
					return 0;
				n = std::min(n, m);
			}
			L.perSm[slot] = n > 0 ? n : 1;
		}
		sms = L.sms;
		perSm = L.perSm[slot];
	}
	if (ctasPerSm > 0 && ctasPerSm < perSm)
		perSm = ctasPerSm;
	const int ctasNeeded = (nblocks + kWarpsPerCta - 1) / kWarpsPerCta;
	const int g = sms * perSm;
	return ctasNeeded < g ? ctasNeeded : g;
}

int GridFor(int nblocks, const nebc7_settings& s)
{
	return GridForSlot(nblocks, VariantSlot(s));
}

/* The launch description of one texture. */
Job SingleJob(uint8_t* dst, const uint8_t* bgra, const uint8_t* mask, long long stride, int blocksW, int nblocks,
	const nebc7_settings& s, BlockResult* results, int* counter, int* status)
{
	Job job;
	job.tex = nullptr;
	job.single.dst = dst;
	job.single.bgra = bgra;
	job.single.mask = mask;
	job.single.stride = stride;
	job.single.blocksW = blocksW;
	job.single.nblocks = nblocks;
	job.single.first = 0;
	job.single.denoise = s.denoise;
	job.single.id = 0;
	job.single.results = nullptr;
	job.single.remaining = nullptr;
	job.single.doneFlag = nullptr;
	job.single.P = MakeParams(s);
	job.ntex = 1;
	job.total = nblocks;
	job.results = results;
	job.counter = counter;
	job.status = status;
	job.order = nullptr;
	return job;
}

/* Scratch of one encode, in 256-byte aligned pieces: the work-queue head,
   status word and reduced sums (256 bytes); the block-order histogram and
   cursors (2 KB); the block order (an int per block) and buckets (a byte per
   block); one BlockResult per block when sums are wanted.  The first
   kScratchZeroed bytes must be zero before a launch. */
constexpr size_t kScratchZeroed = 256 + 2048;

constexpr size_t ScratchAlign(size_t v) { return (v + 255) & ~size_t(255); }

constexpr size_t EncodeScratchBytes(int nblocks, bool wantSums)
{
	return kScratchZeroed + ScratchAlign(size_t(nblocks) * 4) + ScratchAlign(size_t(nblocks)) +
		(wantSums ? size_t(nblocks) * sizeof(BlockResult) : 0) + 64;
}

/* Pieces of a scratch laid out by EncodeScratchBytes. */
struct EncodeScratch
{
	int* counter;
	int* status;
	long long* sums;
	double* ssums;
	int* hist;
	int* cursor;
	int* order;
	uint8_t* bucket;
	BlockResult* results;
};

EncodeScratch SplitScratch(uint8_t* scratch, int nblocks, bool wantSums)
{
	EncodeScratch e;
	e.counter = (int*)scratch;
	e.status = e.counter + 1;
	e.sums = (long long*)(scratch + 64);
	e.ssums = (double*)(scratch + 128);
	e.hist = (int*)(scratch + 256);
	e.cursor = e.hist + 256;
	e.order = (int*)(scratch + kScratchZeroed);
	e.bucket = scratch + kScratchZeroed + ScratchAlign(size_t(nblocks) * 4);
	e.results = wantSums ? (BlockResult*)(e.bucket + ScratchAlign(size_t(nblocks))) : nullptr;
	return e;
}

/* The refining variants take a texture's blocks widest pixel range first
   (KBlockBuckets); the draft-only ones, whose blocks cost about the same,
   in raster order. */
bool OrdersBlocks(const nebc7_settings& s)
{
	return s.doNormal && s.doDraft != 2;
}

/* Enqueues the block order of one texture into e.order (e's zeroed head
   must already be zero on the stream). */
cudaError_t EnqueueBlockOrder(const uint8_t* bgra, long long stride, int blocksW, int nblocks, const EncodeScratch& e,
	cudaStream_t stream)
{
	const int tb = 256;
	const int grid = (nblocks + tb - 1) / tb;
	KBlockBuckets<<<grid, tb, 0, stream>>>(bgra, stride, blocksW, nblocks, e.bucket, e.hist);
	KBlockOrder<<<grid, tb, 0, stream>>>(e.bucket, nblocks, e.hist, e.cursor, e.order);
	return cudaGetLastError();
}

/* Scratch of one encode launch: the staged form adds its per-block records
   after the EncodeScratchBytes pieces. */
size_t LaunchScratchBytes(int nblocks, bool wantSums, const nebc7_settings& s)
{
	const size_t base = (EncodeScratchBytes(nblocks, wantSums) + 255) & ~size_t(255);
	return SlotStaged(VariantSlot(s)) ? base + StagedScratchBytes(nblocks) : base;
}

/* Launches the encode of `job` with instantiation `slot`: the staged form
   when the slot has one and `staged` (StagedScratchBytes(job.total) bytes,
   256-byte aligned) is given, else the single kernel. */
cudaError_t LaunchSlot(int slot, int grid, cudaStream_t stream, const Job& job, const LevelTables& T0, const LevelTables& T1,
	uint8_t* staged)
{
	if (staged && kVariants[slot].staged)
	{
		const Stages sg = SplitStaged(staged, job.total);
		const cudaError_t e = cudaMemsetAsync(staged, 0, kStagedZeroed, stream);
		if (e != cudaSuccess)
			return e;
		return kVariants[slot].staged(grid, stream, job, sg, T0, T1);
	}
	return kVariants[slot].launch(grid, stream, job, T0, T1);
}

/* Enqueues one encode.  `scratchIn` (LaunchScratchBytes bytes, 256-byte
   aligned) is used when given, otherwise the scratch is taken from the
   stream-ordered allocator. */
int LaunchEncode(uint8_t* dst, const uint8_t* bgra, const uint8_t* mask, long long stride, int blocksW, int nblocks,
	const nebc7_settings& s, int64_t* errs, double* ssim, cudaStream_t stream, uint8_t* scratchIn = nullptr)
{
	if (nblocks <= 0)
	{
		if (errs)
			errs[0] = errs[1] = 0;
		if (ssim)
			ssim[0] = ssim[1] = 0;
		return NEBC7_OK;
	}
	int dev = 0;
	CK(cudaGetDevice(&dev));
	const LevelTables* T = nullptr;
	if (int e = BuildTables(dev, s.denoise, &T))
		return e;

	const bool wantSums = errs || ssim;
	uint8_t* scratch = scratchIn;
	if (!scratch && cudaMallocAsync((void**)&scratch, LaunchScratchBytes(nblocks, wantSums, s), stream) != cudaSuccess)
		return SetError(NEBC7_ENOMEM);
	const EncodeScratch e = SplitScratch(scratch, nblocks, wantSums);
	int* status = e.status;
	long long* sums = e.sums;
	double* ssums = e.ssums;
	BlockResult* results = e.results;
	CK(cudaMemsetAsync(scratch, 0, kScratchZeroed, stream));

	Job job = SingleJob(dst, bgra, mask, stride, blocksW, nblocks, s, results, e.counter, status);
	if (OrdersBlocks(s))
	{
		CK(EnqueueBlockOrder(bgra, stride, blocksW, nblocks, e, stream));
		job.order = e.order;
	}
	const int grid = GridFor(nblocks, s);
	if (grid <= 0)
	{
		if (!scratchIn)
			cudaFreeAsync(scratch, stream);
		return SetError(NEBC7_ECUDA);
	}
	const int slot = VariantSlot(s);
	uint8_t* staged = SlotStaged(slot) ? scratch + ((EncodeScratchBytes(nblocks, wantSums) + 255) & ~size_t(255)) : nullptr;
	CK(LaunchSlot(slot, grid, stream, job, *T, *T, staged));

	int rc = NEBC7_OK;
	if (wantSums)
	{
		KReduceResults<<<1, 256, 0, stream>>>(results, nblocks, sums, ssums);
		long long hs[2];
		double hq[2];
		int hstatus = 0;
		CK(cudaMemcpyAsync(hs, sums, sizeof(hs), cudaMemcpyDeviceToHost, stream));
		CK(cudaMemcpyAsync(hq, ssums, sizeof(hq), cudaMemcpyDeviceToHost, stream));
		CK(cudaMemcpyAsync(&hstatus, status, sizeof(int), cudaMemcpyDeviceToHost, stream));
		CK(cudaStreamSynchronize(stream));
		if (errs)
		{
			errs[0] = hs[0];
			errs[1] = hs[1];
		}
		if (ssim)
		{
			ssim[0] = hq[0];
			ssim[1] = hq[1];
		}
		if (hstatus)
			rc = SetError(NEBC7_ELIMIT);
	}
	if (!scratchIn)
		CK(cudaFreeAsync(scratch, stream));
	return rc;
}

/* ---- staging for the host-buffer entries ------------------------------- */

/* One staging slot: a device buffer that only grows and a stream of its own.
   Concurrent host calls (the reference's worker threads) each take a free
   slot, so their copies and kernels overlap; slots live for the process. */
struct HostSlot
{
	int device;
	cudaStream_t stream;
	uint8_t* buf;
	size_t cap;
};

std::mutex gSlotMutex;
std::vector<HostSlot*> gFreeSlots;

HostSlot* AcquireSlot(int dev)
{
	{
		std::lock_guard<std::mutex> lock(gSlotMutex);
		for (size_t i = 0; i < gFreeSlots.size(); i++)
			if (gFreeSlots[i]->device == dev)
			{
				HostSlot* h = gFreeSlots[i];
				gFreeSlots.erase(gFreeSlots.begin() + i);
				return h;
			}
	}
	HostSlot* h = new HostSlot{ dev, nullptr, nullptr, 0 };
	if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
	{
		delete h;
		return nullptr;
	}
	return h;
}

void ReleaseSlot(HostSlot* h)
{
	std::lock_guard<std::mutex> lock(gSlotMutex);
	gFreeSlots.push_back(h);
}

bool ReserveSlot(HostSlot* h, size_t bytes)
{
	if (bytes <= h->cap)
		return true;
	if (h->buf)
	{
		cudaStreamSynchronize(h->stream);
		cudaFree(h->buf);
		h->buf = nullptr;
		h->cap = 0;
	}
	const size_t want = bytes + bytes / 4;
	if (cudaMalloc((void**)&h->buf, want) != cudaSuccess)
		return false;
	h->cap = want;
	return true;
}

inline size_t Align256(size_t v) { return (v + 255) & ~size_t(255); }

/* ---- IBc7Core adapter ------------------------------------------------- */

void CoreInitTables(bool doDraft, bool doNormal, bool doSlow, bool linearData)
{
	gCore.doDraft = doDraft;
	gCore.doNormal = doNormal;
	gCore.doSlow = doSlow;
	gCore.linearData = linearData;
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess)
	{
		SetError(NEBC7_ECUDA);
		return;
	}
	const LevelTables* T = nullptr;
	BuildTables(dev, gCore.denoise, &T);
}

/* Gathers the items' cells and masks into contiguous 64-byte blocks, encodes
   them in one launch and scatters the blocks back (src/Bc7Core.cpp:1936). */
void CoreCompress(const WorkerItem* begin, const WorkerItem* end, int stride, int64_t* pErrorAlpha, int64_t* pErrorColor, BlockSSIM* pssim)
{
	const int n = int(end - begin);
	if (n <= 0)
		return;
	std::vector<uint8_t> cells(size_t(n) * 64), masks(size_t(n) * 64), io(size_t(n) * 16);
	for (int i = 0; i < n; i++)
	{
		for (int r = 0; r < 4; r++)
		{
			memcpy(&cells[size_t(i) * 64 + r * 16], begin[i]._Cell + size_t(r) * stride, 16);
			memcpy(&masks[size_t(i) * 64 + r * 16], begin[i]._Mask + size_t(r) * stride, 16);
		}
		memcpy(&io[size_t(i) * 16], begin[i]._Output, 16);
	}
	int64_t e[2] = { 0, 0 };
	double q[2] = { 0, 0 };
	if (nebc7_encode_blocks_host(cells.data(), masks.data(), io.data(), n, &gCore, e, q) != NEBC7_OK)
		return;
	for (int i = 0; i < n; i++)
		memcpy(begin[i]._Output, &io[size_t(i) * 16], 16);
	*pErrorAlpha += e[0];
	*pErrorColor += e[1];
	pssim->Alpha += q[0];
	pssim->Color += q[1];
}

void CoreDecompress(const WorkerItem* begin, const WorkerItem* end, int stride, int64_t* pErrorAlpha, int64_t* pErrorColor, BlockSSIM* pssim)
{
	(void)pErrorAlpha;
	(void)pErrorColor;
	(void)pssim;
	const int n = int(end - begin);
	if (n <= 0)
		return;
	std::vector<uint8_t> blocks(size_t(n) * 16), bgra(size_t(n) * 64);
	for (int i = 0; i < n; i++)
		memcpy(&blocks[size_t(i) * 16], begin[i]._Output, 16);
	if (nebc7_decode_blocks_host(blocks.data(), bgra.data(), n) != NEBC7_OK)
		return;
	for (int i = 0; i < n; i++)
		for (int r = 0; r < 4; r++)
			memcpy(begin[i]._Cell + size_t(r) * stride, &bgra[size_t(i) * 64 + r * 16], 16);
}

int CoreWeightAlpha()
{
	return gCore.linearData ? 1 : 1000;
}

int CoreWeightColor()
{
	return gCore.linearData ? 3 : 715 + 213 + 72;
}

} // namespace

/* ---- batches ------------------------------------------------------------ */

namespace {

/* Relative cost of one block by preset (measured block throughput on the
   1024x1024 and 2048x2048 workloads: draft 1, default 11, precise 400,
   /slow 480, /data 7200); orders a batch's queue longest first. */
double BlockCost(const nebc7_settings& s)
{
	if (!s.doNormal || s.doDraft == 2)
		return 1.0;
	if (s.linearData)
		return 7200.0;
	if (s.doSlow)
		return 480.0;
	if (!s.denoise || s.denoiseStep == 0)
		return 400.0;
	return 11.0;
}

/* Block-order scratch of a launch of n blocks: histogram and cursors
   (2 KB, zeroed per launch), a bucket byte and an order entry per block. */
size_t OrderScratchBytes(int n)
{
	return 2048 + ((size_t(n) + 255) & ~size_t(255)) + ((size_t(n) * 4 + 255) & ~size_t(255));
}

struct BatchGroup
{
	int slot;                 /* kernel instantiation */
	int firstTex, ntex;       /* entries of the schedule's texture table */
	int queueBase;            /* offset of its queue positions in the results */
	int total;                /* blocks */
	int grid;
	long long stagedOff;      /* its staged-encode records in the batch's staged area, or -1 */
	long long orderOff;       /* its block-order scratch in the batch's order area */
};

struct BatchSchedule
{
	std::vector<TexDesc> table;      /* host copy, groups contiguous */
	std::vector<BatchGroup> groups;
	TexDesc* dTable = nullptr;       /* device copy */
	cudaGraphExec_t graph = nullptr;
	size_t stagedBytes = 0;          /* staged-encode records of all its groups */
	size_t orderBytes = 0;           /* block-order scratch of all its groups */
};

} // namespace

struct nebc7_batch
{
	int device = 0;
	bool fromScratch = false;
	std::vector<nebc7_texture> tex;
	int totalBlocks = 0;
	BatchSchedule sched[2];          /* 0: one mixed launch; 1: one launch per preset group */
	int chosen = 0;
	uint8_t* dmem = nullptr;         /* counters, results, sums */
	uint8_t* stagedArea = nullptr;   /* per-group records of the staged encodes */
	uint8_t* orderArea = nullptr;    /* per-group block orders */
	int* counters = nullptr;
	BlockResult* results = nullptr;
	long long* errs = nullptr;
	double* ssims = nullptr;
	cudaStream_t cap = nullptr;      /* capture stream */
	std::vector<cudaStream_t> side;  /* concurrent preset groups */
	std::vector<cudaEvent_t> ev;     /* fork / join */
	const LevelTables* T[2] = { nullptr, nullptr };
	/* the plan's knobs besides the schedule: the staged form of the groups
	   that have one, and the resident CTAs per SM (0: the occupancy) */
	int staged = 1;
	int ctasPerSm = 0;
	struct Trial
	{
		int schedule, staged, ctasPerSm;
		float ms;
	};
	std::vector<Trial> trials;   /* the last tuning's measurements */
};

namespace {

/* Builds schedule `which` of batch b: the texture table in queue order and
   its launch groups. */
void BuildSchedule(nebc7_batch* b, int which)
{
	BatchSchedule& S = b->sched[which];
	const int n = int(b->tex.size());
	std::vector<int> order(n);
	for (int i = 0; i < n; i++)
		order[i] = i;
	std::vector<double> cost(n);
	std::vector<int> slot(n);
	for (int i = 0; i < n; i++)
	{
		const nebc7_texture& t = b->tex[i];
		cost[i] = BlockCost(t.settings) * double(t.w / 4) * double(t.h / 4);
		slot[i] = which == 0 ? kVariantMixed : VariantSlot(t.settings);
	}
	/* group by instantiation (mixed: one group), longest first within it */
	std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
		if (slot[x] != slot[y])
			return slot[x] < slot[y];
		return cost[x] > cost[y];
	});
	S.table.clear();
	S.groups.clear();
	int queue = 0;
	for (int j = 0; j < n; j++)
	{
		const int i = order[j];
		const nebc7_texture& t = b->tex[i];
		if (S.groups.empty() || S.groups.back().slot != slot[i])
		{
			BatchGroup g;
			g.slot = slot[i];
			g.firstTex = int(S.table.size());
			g.ntex = 0;
			g.queueBase = queue;
			g.total = 0;
			g.grid = 0;
			g.stagedOff = -1;
			g.orderOff = 0;
			S.groups.push_back(g);
		}
		BatchGroup& g = S.groups.back();
		TexDesc d;
		d.dst = t.d_dst;
		d.bgra = t.d_bgra;
		d.mask = t.d_mask;
		d.stride = t.stride;
		d.blocksW = t.w / 4;
		d.nblocks = (t.w / 4) * (t.h / 4);
		d.first = g.total;
		d.denoise = t.settings.denoise;
		d.id = i;
		d.results = nullptr;
		d.remaining = nullptr;
		d.doneFlag = nullptr;
		d.P = MakeParams(t.settings);
		S.table.push_back(d);
		g.ntex++;
		g.total += d.nblocks;
		queue += d.nblocks;
	}
	long long off = 0, ooff = 0;
	for (BatchGroup& g : S.groups)
	{
		g.grid = GridForSlotCap(g.total, g.slot, b->ctasPerSm);
		g.orderOff = ooff;
		ooff += (long long)OrderScratchBytes(g.total);
		g.stagedOff = -1;
		if (SlotStaged(g.slot) && g.total > 0)
		{
			g.stagedOff = off;
			off += (long long)((StagedScratchBytes(g.total) + 255) & ~size_t(255));
		}
	}
	S.stagedBytes = size_t(off);
	S.orderBytes = size_t(ooff);
}

/* Enqueues schedule `which` on stream st (capturable): clears the outputs
   if asked, zeroes the queue heads, launches the groups (concurrently on
   side streams when there are several) and reduces the per-texture sums. */
int EnqueueSchedule(nebc7_batch* b, int which, cudaStream_t st)
{
	BatchSchedule& S = b->sched[which];
	if (b->fromScratch)
		for (const nebc7_texture& t : b->tex)
			CK(cudaMemsetAsync(t.d_dst, 0, size_t(t.w / 4) * (t.h / 4) * 16, st));
	CK(cudaMemsetAsync(b->counters, 0, sizeof(int) * 2 * S.groups.size(), st));
	const int ng = int(S.groups.size());
	if (ng > 1)
	{
		CK(cudaEventRecord(b->ev[0], st));
		for (int g = 1; g < ng; g++)
			CK(cudaStreamWaitEvent(b->side[g - 1], b->ev[0], 0));
	}
	for (int g = 0; g < ng; g++)
	{
		const BatchGroup& G = S.groups[g];
		if (G.total == 0 || G.grid <= 0)
			continue;
		Job job;
		job.tex = S.dTable + G.firstTex;
		job.ntex = G.ntex;
		job.total = G.total;
		job.results = b->results + G.queueBase;
		job.counter = b->counters + 2 * g;
		job.status = b->counters + 2 * g + 1;
		job.order = nullptr;
		job.single = S.table[G.firstTex];
		const cudaStream_t gs = g == 0 ? st : b->side[g - 1];
		/* the group's blocks most expensive preset first, widest pixel range
		   first within a preset (per-texture sums are by block, unchanged) */
		uint8_t* oa = b->orderArea + G.orderOff;
		int* hist = (int*)oa;
		uint8_t* bucket = oa + 2048;
		int* order = (int*)(bucket + ((size_t(G.total) + 255) & ~size_t(255)));
		CK(cudaMemsetAsync(hist, 0, 2048, gs));
		{
			const int tb = 256, ob = (G.total + tb - 1) / tb;
			KJobBuckets<<<ob, tb, 0, gs>>>(job.tex, job.ntex, G.total, bucket, hist);
			KBlockOrder<<<ob, tb, 0, gs>>>(bucket, G.total, hist, hist + 256, order);
			CK(cudaGetLastError());
		}
		job.order = order;
		CK(LaunchSlot(G.slot, G.grid, gs, job, *b->T[0], *b->T[1],
			(b->staged && G.stagedOff >= 0) ? b->stagedArea + G.stagedOff : nullptr));
	}
	if (ng > 1)
	{
		for (int g = 1; g < ng; g++)
		{
			CK(cudaEventRecord(b->ev[g], b->side[g - 1]));
			CK(cudaStreamWaitEvent(st, b->ev[g], 0));
		}
	}
	for (int g = 0; g < ng; g++)
	{
		const BatchGroup& G = S.groups[g];
		if (G.ntex)
		{
			/* per-texture sums over the group's queue positions */
			KReduceTextures<<<G.ntex, 256, 0, st>>>(b->results + G.queueBase, S.dTable + G.firstTex, b->errs, b->ssims);
			CK(cudaGetLastError());
		}
	}
	return NEBC7_OK;
}

/* Captures schedule `which` into a CUDA graph (once). */
int GraphFor(nebc7_batch* b, int which, cudaGraphExec_t* out)
{
	BatchSchedule& S = b->sched[which];
	if (!S.graph)
	{
		cudaGraph_t g = nullptr;
		CK(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
		const int rc = EnqueueSchedule(b, which, b->cap);
		const cudaError_t e = cudaStreamEndCapture(b->cap, &g);
		if (rc != NEBC7_OK || e != cudaSuccess)
		{
			if (g)
				cudaGraphDestroy(g);
			return SetError(rc != NEBC7_OK ? rc : NEBC7_ECUDA);
		}
		const cudaError_t ie = cudaGraphInstantiate(&S.graph, g, 0);
		cudaGraphDestroy(g);
		if (ie != cudaSuccess)
		{
			S.graph = nullptr;
			return SetError(NEBC7_ECUDA);
		}
	}
	*out = S.graph;
	return NEBC7_OK;
}

/* Sets the plan's knobs; a change of the staged form or of the grid drops
   the captured graphs, which the next launch captures again. */
int ApplyPlan(nebc7_batch* b, int schedule, int staged, int ctasPerSm)
{
	if (staged != b->staged || ctasPerSm != b->ctasPerSm)
	{
		b->staged = staged;
		b->ctasPerSm = ctasPerSm;
		for (BatchSchedule& S : b->sched)
		{
			if (S.graph)
				cudaGraphExecDestroy(S.graph);
			S.graph = nullptr;
			for (BatchGroup& g : S.groups)
			{
				g.grid = GridForSlotCap(g.total, g.slot, ctasPerSm);
				if (g.grid <= 0 && g.total > 0)
					return SetError(NEBC7_ECUDA);
			}
		}
	}
	b->chosen = schedule;
	return NEBC7_OK;
}

void FreeBatch(nebc7_batch* b)
{
	if (!b)
		return;
	cudaSetDevice(b->device);
	for (BatchSchedule& S : b->sched)
	{
		if (S.graph)
			cudaGraphExecDestroy(S.graph);
		cudaFree(S.dTable);
	}
	for (cudaStream_t s : b->side)
		cudaStreamDestroy(s);
	for (cudaEvent_t e : b->ev)
		cudaEventDestroy(e);
	if (b->cap)
		cudaStreamDestroy(b->cap);
	cudaFree(b->dmem);
	cudaFree(b->stagedArea);
	cudaFree(b->orderArea);
	delete b;
}

} // namespace

/* ---- serving ------------------------------------------------------------- */

namespace {

double NowSeconds()
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct ServerRequest
{
	const uint8_t* bgra;
	const uint8_t* mask;
	long long stride;
	int w, h;
	nebc7_settings settings;
	uint8_t* dst;
	double tSubmit = 0, tLaunch = 0, tDone = 0;
	int slot = -1;               /* the launch slot that ran it */
	long long launch = -1;       /* the server's launch sequence number */
	int state = 0;               /* 0 queued, 1 admitted, 2 on the device, 3 done, < 0 error code */
	size_t off = 0, bytes = 0;   /* its part of the arena */
	int64_t errs[2] = { 0, 0 };
	double ssim[2] = { 0, 0 };
};

/* One launch slot: a stream, the batch's texture table and sums. */
struct ServerSlot
{
	cudaStream_t stream = nullptr;   /* the batch's kernel */
	cudaStream_t copies = nullptr;   /* each request's sums and blocks, as it completes */
	cudaEvent_t done = nullptr;      /* end of the kernel */
	bool busy = false;
	std::vector<int64_t> reqs;
	std::vector<int> stage;          /* per request: 0 running, 1 copies enqueued, 2 done */
	std::vector<cudaEvent_t> copied; /* per request: end of its copies */
	TexDesc* hTable = nullptr;       /* pinned */
	TexDesc* dTable = nullptr;
	int* hRemaining = nullptr;       /* pinned staging of the block counts */
	int* dRemaining = nullptr;
	int* hFlags = nullptr;           /* host memory the kernel writes (mapped) */
	int* dFlags = nullptr;
	long long* hSums = nullptr;      /* pinned: 2 errs + 2 ssim (as bits) per request */
	long long* dSums = nullptr;
	int* dCounter = nullptr;
	uint8_t* staged = nullptr;       /* records of a staged launch of up to stagedCap blocks */
	int stagedCap = 0;
};

/* First-fit allocator over the arena (offsets, host bookkeeping only). */
struct ArenaAllocator
{
	std::map<size_t, size_t> free;   /* offset -> size */
	size_t inUse = 0, peak = 0;

	void Init(size_t bytes) { free.clear(); free[0] = bytes; }

	bool Alloc(size_t bytes, size_t* off)
	{
		for (auto it = free.begin(); it != free.end(); ++it)
			if (it->second >= bytes)
			{
				*off = it->first;
				const size_t rest = it->second - bytes;
				const size_t at = it->first + bytes;
				free.erase(it);
				if (rest)
					free[at] = rest;
				inUse += bytes;
				peak = std::max(peak, inUse);
				return true;
			}
		return false;
	}

	void Free(size_t off, size_t bytes)
	{
		inUse -= bytes;
		auto it = free.emplace(off, bytes).first;
		auto next = std::next(it);
		if (next != free.end() && it->first + it->second == next->first)
		{
			it->second += next->second;
			free.erase(next);
		}
		if (it != free.begin())
		{
			auto prev = std::prev(it);
			if (prev->first + prev->second == it->first)
			{
				prev->second += it->second;
				free.erase(it);
			}
		}
	}
};

} // namespace

struct nebc7_server
{
	nebc7_server_config cfg{};
	int device = 0;
	uint8_t* arena = nullptr;
	ArenaAllocator alloc;
	std::mutex mu;
	std::condition_variable cv;       /* wakes waiters on completion */
	std::condition_variable work;     /* wakes the scheduler */
	std::deque<int64_t> queued;
	std::deque<int64_t> admitted;
	std::unordered_map<int64_t, ServerRequest> reqs;
	int64_t nextId = 0;
	std::vector<ServerSlot> slots;
	std::thread worker;
	bool stop = false;
	const LevelTables* T[2] = { nullptr, nullptr };
	long long launches = 0, completed = 0, failed = 0;
	double t0 = 0;                    /* creation time, origin of the request times */
};

namespace {

/* Arena bytes a block needs at least (its pixels, output and result), and
   the most blocks one staged launch of the request loop holds records for. */
constexpr size_t kServerBlockBytes = 64 + 16 + sizeof(BlockResult);
constexpr int kServerStagedBlocks = 1 << 22;

/* A request whose preset runs the full searches on most blocks (the
   precise preset, /slow, /data). */
bool HeavyRequest(const ServerRequest& r)
{
	return BlockCost(r.settings) >= 400.0;
}

size_t RequestBytes(const ServerRequest& r)
{
	const size_t nb = size_t(r.w / 4) * (r.h / 4);
	const size_t img = size_t(r.w) * 4 * r.h;
	return Align256(img) + (r.mask ? Align256(img) : 0) + Align256(nb * 16) + Align256(nb * sizeof(BlockResult));
}

/* Enqueues one batch of admitted requests on a free slot: copies in,
   clears the outputs, one mixed-preset persistent launch over the batch,
   per-request sums, copies out; the slot's event marks the end. */
int LaunchServerBatch(nebc7_server* sv, ServerSlot& slot, std::vector<int64_t>& batch)
{
	const cudaStream_t st = slot.stream;
	/* shortest expected work first: cheap requests finish (and return) while
	   the expensive ones still run */
	std::stable_sort(batch.begin(), batch.end(), [&](int64_t x, int64_t y) {
		const ServerRequest& a = sv->reqs[x];
		const ServerRequest& b = sv->reqs[y];
		return BlockCost(a.settings) * double(a.w) * a.h < BlockCost(b.settings) * double(b.w) * b.h;
	});
	int total = 0;
	for (size_t k = 0; k < batch.size(); k++)
	{
		ServerRequest& r = sv->reqs[batch[k]];
		uint8_t* base = sv->arena + r.off;
		const size_t nb = size_t(r.w / 4) * (r.h / 4);
		const size_t img = size_t(r.w) * 4 * r.h;
		uint8_t* dImg = base;
		uint8_t* dMask = r.mask ? base + Align256(img) : nullptr;
		uint8_t* dDst = base + Align256(img) + (r.mask ? Align256(img) : 0);
		BlockResult* dRes = (BlockResult*)(dDst + Align256(nb * 16));
		CK(cudaMemcpy2DAsync(dImg, size_t(r.w) * 4, r.bgra, size_t(r.stride), size_t(r.w) * 4, size_t(r.h), cudaMemcpyHostToDevice, st));
		if (r.mask)
			CK(cudaMemcpy2DAsync(dMask, size_t(r.w) * 4, r.mask, size_t(r.stride), size_t(r.w) * 4, size_t(r.h), cudaMemcpyHostToDevice, st));
		CK(cudaMemsetAsync(dDst, 0, nb * 16, st));
		TexDesc& d = slot.hTable[k];
		d.dst = dDst;
		d.bgra = dImg;
		d.mask = dMask;
		d.stride = (long long)r.w * 4;
		d.blocksW = r.w / 4;
		d.nblocks = int(nb);
		d.first = total;
		d.denoise = r.settings.denoise;
		d.id = int(k);
		d.results = dRes;
		d.remaining = slot.dRemaining + k;
		d.doneFlag = slot.dFlags + k;
		d.P = MakeParams(r.settings);
		total += int(nb);
		slot.hRemaining[k] = int(nb);
		reinterpret_cast<volatile int*>(slot.hFlags)[k] = 0;
	}
	CK(cudaMemcpyAsync(slot.dTable, slot.hTable, sizeof(TexDesc) * batch.size(), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(slot.dRemaining, slot.hRemaining, sizeof(int) * batch.size(), cudaMemcpyHostToDevice, st));
	CK(cudaMemsetAsync(slot.dCounter, 0, 2 * sizeof(int), st));
	Job job;
	job.tex = slot.dTable;
	job.ntex = int(batch.size());
	job.total = total;
	job.results = nullptr;
	job.counter = slot.dCounter;
	job.status = slot.dCounter + 1;
	job.order = nullptr;
	job.single = slot.hTable[0];
	const int grid = GridForSlot(total, kVariantMixed);
	if (grid <= 0)
		return SetError(NEBC7_ECUDA);
	/* a batch of heavy requests takes the staged form (one kernel per pass);
	   a batch of light ones the single kernel, whose blocks and so whose
	   requests finish as they go */
	bool heavy = total <= slot.stagedCap;
	for (int64_t id : batch)
		heavy = heavy && HeavyRequest(sv->reqs[id]);
	CK(LaunchSlot(kVariantMixed, grid, st, job, *sv->T[0], *sv->T[1], heavy ? slot.staged : nullptr));
	CK(cudaEventRecord(slot.done, st));
	slot.stage.assign(batch.size(), 0);
	return NEBC7_OK;
}

/* Request k of a busy slot has all its blocks: reduce its sums and copy its
   blocks and sums back on the slot's copy stream. */
int ReturnServerRequest(nebc7_server* sv, ServerSlot& slot, size_t k)
{
	const cudaStream_t cs = slot.copies;
	const int cap = sv->cfg.max_batch;
	ServerRequest& r = sv->reqs[slot.reqs[k]];
	const size_t nb = size_t(r.w / 4) * (r.h / 4);
	KReduceTextures<<<1, 256, 0, cs>>>(nullptr, slot.dTable + k, slot.dSums, (double*)(slot.dSums + 2 * cap));
	CK(cudaGetLastError());
	CK(cudaMemcpyAsync(slot.hSums + 2 * k, slot.dSums + 2 * k, 2 * sizeof(long long), cudaMemcpyDeviceToHost, cs));
	CK(cudaMemcpyAsync(slot.hSums + 2 * cap + 2 * k, slot.dSums + 2 * cap + 2 * k, 2 * sizeof(long long),
		cudaMemcpyDeviceToHost, cs));
	CK(cudaMemcpyAsync(r.dst, slot.hTable[k].dst, nb * 16, cudaMemcpyDeviceToHost, cs));
	CK(cudaEventRecord(slot.copied[k], cs));
	return NEBC7_OK;
}

/* Advances the busy slots: returns each request as soon as the kernel has
   flagged all its blocks, completes it when its copies are done (sums,
   times, arena space), and frees a slot once its kernel and all its
   requests are finished.  Called with sv->mu held. */
void FinishServerRequest(nebc7_server* sv, ServerSlot& slot, size_t k, int rc)
{
	const int cap = sv->cfg.max_batch;
	ServerRequest& r = sv->reqs[slot.reqs[k]];
	if (rc == NEBC7_OK)
	{
		r.errs[0] = slot.hSums[2 * k];
		r.errs[1] = slot.hSums[2 * k + 1];
		memcpy(&r.ssim[0], &slot.hSums[2 * cap + 2 * k], sizeof(double));
		memcpy(&r.ssim[1], &slot.hSums[2 * cap + 2 * k + 1], sizeof(double));
		r.state = 3;
		sv->completed++;
	}
	else
	{
		r.state = -rc;
		sv->failed++;
	}
	r.tDone = NowSeconds();
	sv->alloc.Free(r.off, r.bytes);
	slot.stage[k] = 2;
}

bool ReapServer(nebc7_server* sv)
{
	bool any = false;
	for (ServerSlot& slot : sv->slots)
	{
		if (!slot.busy)
			continue;
		const cudaError_t kq = cudaEventQuery(slot.done);
		const bool kernelFailed = kq != cudaSuccess && kq != cudaErrorNotReady;
		bool all = true;
		for (size_t k = 0; k < slot.reqs.size(); k++)
		{
			if (slot.stage[k] == 0)
			{
				if (kernelFailed)
				{
					FinishServerRequest(sv, slot, k, NEBC7_ECUDA);
					any = true;
					continue;
				}
				if (reinterpret_cast<volatile int*>(slot.hFlags)[k] == 1)
				{
					const int rc = ReturnServerRequest(sv, slot, k);
					if (rc != NEBC7_OK)
						FinishServerRequest(sv, slot, k, rc);
					else
						slot.stage[k] = 1;
					any = true;
				}
			}
			if (slot.stage[k] == 1)
			{
				const cudaError_t q = cudaEventQuery(slot.copied[k]);
				if (q != cudaErrorNotReady)
				{
					FinishServerRequest(sv, slot, k, q == cudaSuccess ? NEBC7_OK : NEBC7_ECUDA);
					any = true;
				}
			}
			all &= slot.stage[k] == 2;
		}
		if (all && kq != cudaErrorNotReady)
		{
			slot.reqs.clear();
			slot.busy = false;
			any = true;
		}
	}
	return any;
}

/* The scheduler: admits queued requests in arrival order while the arena
   has room, and starts a batch of admitted requests on every free slot,
   so that new requests join the device while earlier batches run. */
void ServerLoop(nebc7_server* sv)
{
	cudaSetDevice(sv->device);
	std::unique_lock<std::mutex> lock(sv->mu);
	for (;;)
	{
		bool progress = ReapServer(sv);
		if (progress)
			sv->cv.notify_all();
		while (!sv->queued.empty())
		{
			ServerRequest& r = sv->reqs[sv->queued.front()];
			if (!sv->alloc.Alloc(r.bytes, &r.off))
				break;
			r.state = 1;
			sv->admitted.push_back(sv->queued.front());
			sv->queued.pop_front();
			progress = true;
		}
		for (ServerSlot& slot : sv->slots)
		{
			if (slot.busy || sv->admitted.empty())
				continue;
			/* the oldest admitted request and, in arrival order, others of its
			   kind (heavy or light presets) up to max_batch requests and, for
			   heavy ones, the staged records' capacity */
			std::vector<int64_t> batch;
			const bool heavy = HeavyRequest(sv->reqs[sv->admitted.front()]);
			long long blocks = 0;
			for (auto it = sv->admitted.begin(); it != sv->admitted.end() && int(batch.size()) < sv->cfg.max_batch;)
			{
				const ServerRequest& r = sv->reqs[*it];
				const long long nb = (long long)(r.w / 4) * (r.h / 4);
				if (HeavyRequest(r) != heavy || (!batch.empty() && heavy && blocks + nb > slot.stagedCap))
				{
					++it;
					continue;
				}
				blocks += nb;
				batch.push_back(*it);
				it = sv->admitted.erase(it);
			}
			const double now = NowSeconds();
			for (int64_t id : batch)
			{
				ServerRequest& r = sv->reqs[id];
				r.state = 2;
				r.tLaunch = now;
				r.slot = int(&slot - sv->slots.data());
				r.launch = sv->launches;
			}
			const int rc = LaunchServerBatch(sv, slot, batch);
			if (rc != NEBC7_OK)
			{
				/* nothing of the batch is known to be in flight: wait for the
				   stream, then fail its requests */
				cudaStreamSynchronize(slot.stream);
				for (int64_t id : batch)
				{
					ServerRequest& r = sv->reqs[id];
					r.state = -rc;
					r.tDone = NowSeconds();
					sv->alloc.Free(r.off, r.bytes);
					sv->failed++;
				}
				sv->cv.notify_all();
				continue;
			}
			slot.reqs = batch;
			slot.busy = true;
			sv->launches++;
			progress = true;
		}
		bool busy = false;
		for (const ServerSlot& slot : sv->slots)
			busy |= slot.busy;
		if (sv->stop && !busy && sv->queued.empty() && sv->admitted.empty())
			break;
		if (!progress)
		{
			/* poll the device while batches run; sleep until a submit otherwise */
			if (busy)
				sv->work.wait_for(lock, std::chrono::microseconds(50));
			else
				sv->work.wait(lock, [&] { return sv->stop || !sv->queued.empty(); });
		}
	}
}

void FreeServer(nebc7_server* sv)
{
	if (!sv)
		return;
	cudaSetDevice(sv->device);
	for (ServerSlot& slot : sv->slots)
	{
		if (slot.stream)
			cudaStreamSynchronize(slot.stream);
		if (slot.copies)
			cudaStreamSynchronize(slot.copies);
		cudaStreamDestroy(slot.stream);
		cudaStreamDestroy(slot.copies);
		cudaEventDestroy(slot.done);
		for (cudaEvent_t e : slot.copied)
			if (e)
				cudaEventDestroy(e);
		cudaFreeHost(slot.hFlags);
		cudaFreeHost(slot.hRemaining);
		cudaFree(slot.dRemaining);
		cudaFreeHost(slot.hTable);
		cudaFreeHost(slot.hSums);
		cudaFree(slot.dTable);
		cudaFree(slot.dSums);
		cudaFree(slot.dCounter);
		cudaFree(slot.staged);
	}
	cudaFree(sv->arena);
	delete sv;
}

} // namespace

/* ---- allocation-free encode -------------------------------------------- */

/* Largest texture nebc7_encode_device_noalloc accepts: 65536 blocks
   (1024x1024 pixels).  Its scratch lives in this fixed device array instead
   of coming from an allocator: 256 bytes for the work-queue head and the
   status word, the block order, then one BlockResult per block for the
   error / SSIM sums (the layout of EncodeScratchBytes). */
constexpr int kNoAllocMaxBlocks = 65536;
constexpr size_t kNoAllocScratchBytes = EncodeScratchBytes(kNoAllocMaxBlocks, true);
/* 2304 + 262144 + 65536 + 65536 * 24 + 64 bytes: about 1.9 MB on every device
   that loads the library */
static_assert(kNoAllocScratchBytes == 1902912, "the documented size of the allocation-free scratch");
static __device__ __align__(256) unsigned char gNoAllocScratch[kNoAllocScratchBytes];

namespace {

std::mutex gNoAllocMutex;
uint8_t* gNoAllocPtr[kMaxDevices] = {};

/* Device address of gNoAllocScratch on `dev`, looked up once per device
   (with that device current) and cached. */
int NoAllocScratch(int dev, uint8_t** out)
{
	if (dev < 0 || dev >= kMaxDevices)
		return SetError(NEBC7_EINVAL);
	std::lock_guard<std::mutex> lock(gNoAllocMutex);
	if (!gNoAllocPtr[dev])
	{
		void* p = nullptr;
		if (cudaGetSymbolAddress(&p, gNoAllocScratch) != cudaSuccess || !p)
			return SetError(NEBC7_ECUDA);
		gNoAllocPtr[dev] = (uint8_t*)p;
	}
	*out = gNoAllocPtr[dev];
	return NEBC7_OK;
}

/* The level tables of `denoise` on `dev` if they were already built, else null. */
const LevelTables* BuiltTables(int dev, int denoise)
{
	std::lock_guard<std::mutex> lock(gMutex);
	if (dev < 0 || dev >= kMaxDevices || !gTables[dev][denoise].built)
		return nullptr;
	return &gTables[dev][denoise].t;
}

} // namespace

extern "C" {

int nebc7_encode_device_noalloc(uint8_t* d_dst, const uint8_t* d_bgra, const uint8_t* d_mask, long long stride, int w,
	int h, const nebc7_settings* settings, void* d_sums, void* stream)
{
	if (int e = ValidateSettings(settings))
		return SetError(e);
	if (w <= 0 || h <= 0 || (w & 3) || (h & 3) || stride < (long long)w * 4 || (stride & 3))
		return SetError(NEBC7_EINVAL);
	if (((uintptr_t)d_dst & 15) || ((uintptr_t)d_bgra & 3) || ((uintptr_t)d_mask & 3) || ((uintptr_t)d_sums & 7))
		return SetError(NEBC7_EINVAL);
	const long long nb = (long long)(w / 4) * (h / 4);
	if (nb > kNoAllocMaxBlocks)
		return SetError(NEBC7_ETOOBIG);
	int dev = 0;
	CK(cudaGetDevice(&dev));
	const LevelTables* T = BuiltTables(dev, settings->denoise);
	if (!T)
		return SetError(NEBC7_EINVAL);   /* nebc7_init_device(denoise) was not called on this device */
	uint8_t* scratch = nullptr;
	if (int e = NoAllocScratch(dev, &scratch))
		return e;

	const int grid = GridFor(int(nb), *settings);
	if (grid <= 0)
		return SetError(NEBC7_ECUDA);

	const cudaStream_t st = (cudaStream_t)stream;
	/* the queue head, status word and block-order counts must start at zero */
	CK(cudaMemsetAsync(scratch, 0, kScratchZeroed, st));
	const EncodeScratch e = SplitScratch(scratch, int(nb), d_sums != nullptr);
	Job job = SingleJob(d_dst, d_bgra, d_mask, stride, w / 4, int(nb), *settings, e.results, e.counter, e.status);
	if (OrdersBlocks(*settings))
	{
		CK(EnqueueBlockOrder(d_bgra, stride, w / 4, int(nb), e, st));
		job.order = e.order;
	}
	CK(kVariants[VariantSlot(*settings)].launch(grid, st, job, *T, *T));
	if (d_sums)
	{
		KReduceResults<<<1, 256, 0, st>>>(job.results, int(nb), (long long*)d_sums, (double*)((uint8_t*)d_sums + 16));
		CK(cudaGetLastError());
	}
	return NEBC7_OK;
}


bool nebc7_GetBc7Core(void* bc7Core)
{
	int count = 0;
	if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0)
		return false;
	IBc7Core* p = reinterpret_cast<IBc7Core*>(bc7Core);
	p->pInitTables = &CoreInitTables;
	p->pDecompress = &CoreDecompress;
	p->pCompress = &CoreCompress;
	p->pGetWeightAlpha = &CoreWeightAlpha;
	p->pGetWeightColor = &CoreWeightColor;
	return true;
}

void nebc7_ProcessTexture(uint8_t* dst, uint8_t* src_bgra, uint8_t* mask_agrb, int stride, int src_w, int src_h,
	PBlockKernel blockKernel, size_t block_size, int64_t* pErrorAlpha, int64_t* pErrorColor, BlockSSIM* pssim)
{
	if (block_size != 16)
	{
		SetError(NEBC7_EINVAL);
		return;
	}
	if (blockKernel == &CoreCompress)
	{
		int64_t e[2] = { 0, 0 };
		double q[2] = { 0, 0 };
		if (nebc7_encode_host(dst, src_bgra, mask_agrb, stride, src_w, src_h, &gCore, e, q) != NEBC7_OK)
			return;
		*pErrorAlpha = e[0];
		*pErrorColor = e[1];
		pssim->Alpha = q[0];
		pssim->Color = q[1];
	}
	else if (blockKernel == &CoreDecompress)
	{
		/* decode every block back into src_bgra (the reference's /debug pass) */
		const int bw = src_w / 4, bh = src_h / 4;
		std::vector<uint8_t> bgra(size_t(bw) * bh * 64);
		if (nebc7_decode_blocks_host(dst, bgra.data(), bw * bh) != NEBC7_OK)
			return;
		for (int k = 0; k < bw * bh; k++)
			for (int r = 0; r < 4; r++)
				memcpy(src_bgra + size_t(k / bw * 4 + r) * stride + size_t(k % bw) * 16, &bgra[size_t(k) * 64 + r * 16], 16);
	}
	else
	{
		SetError(NEBC7_EINVAL);
	}
}

int nebc7_set_preset(int denoise, int denoiseStep)
{
	if ((denoise != 0 && denoise != 1) || denoiseStep < 0 || denoiseStep > 4096)
		return SetError(NEBC7_EINVAL);
	gCore.denoise = denoise;
	gCore.denoiseStep = denoiseStep;
	return NEBC7_OK;
}

int nebc7_last_error(void)
{
	return gLastError;
}

int nebc7_encode_device(uint8_t* d_dst, const uint8_t* d_bgra, const uint8_t* d_mask, long long stride, int w, int h,
	const nebc7_settings* settings, int64_t* errs, double* ssim, void* stream)
{
	if (int e = ValidateSettings(settings))
		return SetError(e);
	if (w <= 0 || h <= 0 || (w & 3) || (h & 3) || stride < (long long)w * 4 || (stride & 3))
		return SetError(NEBC7_EINVAL);
	if (((uintptr_t)d_dst & 15) || ((uintptr_t)d_bgra & 3) || ((uintptr_t)d_mask & 3))
		return SetError(NEBC7_EINVAL);
	const long long nb = (long long)(w / 4) * (h / 4);
	if (nb > 0x7FFFFFFF)
		return SetError(NEBC7_ETOOBIG);
	return LaunchEncode(d_dst, d_bgra, d_mask, stride, w / 4, int(nb), *settings, errs, ssim, (cudaStream_t)stream);
}

int nebc7_encode_host(uint8_t* dst, const uint8_t* bgra, const uint8_t* mask, long long stride, int w, int h,
	const nebc7_settings* settings, int64_t* errs, double* ssim)
{
	if (int e = ValidateSettings(settings))
		return SetError(e);
	if (w <= 0 || h <= 0 || (w & 3) || (h & 3) || stride < (long long)w * 4)
		return SetError(NEBC7_EINVAL);
	const size_t nb = size_t(w / 4) * (h / 4);
	const size_t img = size_t(w) * 4 * h;
	if (nb > size_t(0x7FFFFFFF))
		return SetError(NEBC7_ETOOBIG);
	int dev = 0;
	CK(cudaGetDevice(&dev));
	HostSlot* slot = AcquireSlot(dev);
	if (!slot)
		return SetError(NEBC7_ECUDA);
	const size_t offImg = Align256(nb * 16);
	const size_t offMask = offImg + Align256(img);
	const size_t offScratch = offMask + (mask ? Align256(img) : 0);
	if (!ReserveSlot(slot, offScratch + LaunchScratchBytes(int(nb), true, *settings)))
	{
		ReleaseSlot(slot);
		return SetError(NEBC7_ENOMEM);
	}
	cudaStream_t st = slot->stream;
	uint8_t* dd = slot->buf;
	uint8_t* db = slot->buf + offImg;
	uint8_t* dm = mask ? slot->buf + offMask : nullptr;
	int rc = NEBC7_OK;
	if (cudaMemcpy2DAsync(db, size_t(w) * 4, bgra, size_t(stride), size_t(w) * 4, size_t(h), cudaMemcpyHostToDevice, st) != cudaSuccess ||
		(mask && cudaMemcpy2DAsync(dm, size_t(w) * 4, mask, size_t(stride), size_t(w) * 4, size_t(h), cudaMemcpyHostToDevice, st) != cudaSuccess) ||
		cudaMemcpyAsync(dd, dst, nb * 16, cudaMemcpyHostToDevice, st) != cudaSuccess)
		rc = SetError(NEBC7_ECUDA);
	int64_t e[2];
	double q[2];
	if (rc == NEBC7_OK)
		rc = LaunchEncode(dd, db, dm, (long long)w * 4, w / 4, int(nb), *settings, e, q, st, slot->buf + offScratch);
	if (rc == NEBC7_OK && (cudaMemcpyAsync(dst, dd, nb * 16, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
		cudaStreamSynchronize(st) != cudaSuccess))
		rc = SetError(NEBC7_ECUDA);
	if (rc == NEBC7_OK)
	{
		if (errs)
		{
			errs[0] = e[0];
			errs[1] = e[1];
		}
		if (ssim)
		{
			ssim[0] = q[0];
			ssim[1] = q[1];
		}
	}
	else
		cudaStreamSynchronize(st);
	ReleaseSlot(slot);
	return rc;
}

int nebc7_encode_blocks_host(const uint8_t* cells, const uint8_t* masks, uint8_t* io, int n,
	const nebc7_settings* settings, int64_t* errs, double* ssim)
{
	if (int e = ValidateSettings(settings))
		return SetError(e);
	if (n < 0)
		return SetError(NEBC7_EINVAL);
	if (n == 0)
	{
		if (errs)
			errs[0] = errs[1] = 0;
		if (ssim)
			ssim[0] = ssim[1] = 0;
		return NEBC7_OK;
	}
	/* a column of blocks: stride 16, one block per block row */
	return nebc7_encode_host(io, cells, masks, 16, 4, 4 * n, settings, errs, ssim);
}

int nebc7_decode_device(const uint8_t* d_blocks, uint8_t* d_bgra, long long stride, int w, int h, void* stream)
{
	if (w <= 0 || h <= 0 || (w & 3) || (h & 3) || stride < (long long)w * 4 || (stride & 3) || ((uintptr_t)d_blocks & 15))
		return SetError(NEBC7_EINVAL);
	const long long nb = (long long)(w / 4) * (h / 4);
	const long long threads = nb * 16;
	KDecode<<<unsigned((threads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(d_blocks, d_bgra, stride, w / 4, int(nb));
	CK(cudaGetLastError());
	return NEBC7_OK;
}

int nebc7_decode_blocks_host(const uint8_t* blocks, uint8_t* bgra, int n)
{
	if (n < 0)
		return SetError(NEBC7_EINVAL);
	if (n == 0)
		return NEBC7_OK;
	uint8_t *db = nullptr, *dp = nullptr;
	if (cudaMalloc(&db, size_t(n) * 16) != cudaSuccess || cudaMalloc(&dp, size_t(n) * 64) != cudaSuccess)
	{
		cudaFree(db);
		return SetError(NEBC7_ENOMEM);
	}
	int rc = NEBC7_OK;
	if (cudaMemcpy(db, blocks, size_t(n) * 16, cudaMemcpyHostToDevice) != cudaSuccess)
		rc = SetError(NEBC7_ECUDA);
	if (rc == NEBC7_OK)
		rc = nebc7_decode_device(db, dp, 16, 4, 4 * n, nullptr);
	if (rc == NEBC7_OK && cudaMemcpy(bgra, dp, size_t(n) * 64, cudaMemcpyDeviceToHost) != cudaSuccess)
		rc = SetError(NEBC7_ECUDA);
	cudaFree(db);
	cudaFree(dp);
	return rc;
}

int nebc7_set_pca(int on)
{
	if (on != 0 && on != 1)
		return SetError(NEBC7_EINVAL);
	gPca.store(on);
	return NEBC7_OK;
}

int nebc7_encode_launches(const nebc7_settings* settings)
{
	if (int e = ValidateSettings(settings))
		return -SetError(e);
	const int order = OrdersBlocks(*settings) ? 2 : 0;
	return order + (SlotStaged(VariantSlot(*settings)) ? StagedLaunches() : 1);
}

int nebc7_init_device(int denoise)
{
	if (denoise != 0 && denoise != 1)
		return SetError(NEBC7_EINVAL);
	int dev = 0;
	CK(cudaGetDevice(&dev));
	const LevelTables* T = nullptr;
	return BuildTables(dev, denoise, &T);
}

int nebc7_table_read(int denoise, int which, void* host, long long capacity, long long* bytes)
{
	if ((denoise != 0 && denoise != 1) || which < 0 || which >= kNumLevelTables || !host || !bytes)
		return SetError(NEBC7_EINVAL);
	int dev = 0;
	CK(cudaGetDevice(&dev));
	const LevelTables* T = nullptr;
	if (int e = BuildTables(dev, denoise, &T))
		return e;
	const size_t n = kLevelTableBytes[which];
	*bytes = (long long)n;
	if (capacity < (long long)n)
		return SetError(NEBC7_ETOOBIG);
	CK(cudaMemcpy(host, gTables[dev][denoise].mem[which], n, cudaMemcpyDeviceToHost));
	return NEBC7_OK;
}

int nebc7_batch_create(const nebc7_texture* textures, int n, int flags, nebc7_batch** out)
{
	if (!out || n <= 0 || !textures || (flags & ~NEBC7_BATCH_FROM_SCRATCH))
		return SetError(NEBC7_EINVAL);
	*out = nullptr;
	long long total = 0;
	for (int i = 0; i < n; i++)
	{
		const nebc7_texture& t = textures[i];
		if (int e = ValidateSettings(&t.settings))
			return SetError(e);
		if (t.w <= 0 || t.h <= 0 || (t.w & 3) || (t.h & 3) || t.stride < (long long)t.w * 4 || (t.stride & 3))
			return SetError(NEBC7_EINVAL);
		if (!t.d_dst || !t.d_bgra || ((uintptr_t)t.d_dst & 15) || ((uintptr_t)t.d_bgra & 3) || ((uintptr_t)t.d_mask & 3))
			return SetError(NEBC7_EINVAL);
		total += (long long)(t.w / 4) * (t.h / 4);
	}
	if (total > 0x7FFFFFFF)
		return SetError(NEBC7_ETOOBIG);
	nebc7_batch* b = new nebc7_batch;
	b->fromScratch = (flags & NEBC7_BATCH_FROM_SCRATCH) != 0;
	b->tex.assign(textures, textures + n);
	b->totalBlocks = int(total);
	int rc = NEBC7_OK;
	if (cudaGetDevice(&b->device) != cudaSuccess)
		rc = SetError(NEBC7_ECUDA);
	for (int d = 0; d < 2 && rc == NEBC7_OK; d++)
		rc = BuildTables(b->device, d, &b->T[d]);
	if (rc == NEBC7_OK)
	{
		BuildSchedule(b, 0);
		BuildSchedule(b, 1);
		const size_t ng = std::max(b->sched[0].groups.size(), b->sched[1].groups.size());
		const size_t offRes = 256 + ((sizeof(int) * 2 * ng + 255) & ~size_t(255));
		const size_t offErr = offRes + ((size_t(total) * sizeof(BlockResult) + 255) & ~size_t(255));
		const size_t bytes = offErr + size_t(n) * 4 * sizeof(long long);
		const size_t stagedBytes = std::max(b->sched[0].stagedBytes, b->sched[1].stagedBytes);
		const size_t orderBytes = std::max(b->sched[0].orderBytes, b->sched[1].orderBytes);
		if (cudaMalloc((void**)&b->dmem, bytes) != cudaSuccess ||
			(stagedBytes && cudaMalloc((void**)&b->stagedArea, stagedBytes) != cudaSuccess) ||
			cudaMalloc((void**)&b->orderArea, orderBytes) != cudaSuccess)
			rc = SetError(NEBC7_ENOMEM);
		else
		{
			b->counters = (int*)(b->dmem + 256);
			b->results = (BlockResult*)(b->dmem + offRes);
			b->errs = (long long*)(b->dmem + offErr);
			b->ssims = (double*)(b->errs + 2 * n);
		}
		for (int w = 0; w < 2 && rc == NEBC7_OK; w++)
		{
			BatchSchedule& S = b->sched[w];
			for (const BatchGroup& g : S.groups)
				if (g.grid <= 0 && g.total > 0)
					rc = SetError(NEBC7_ECUDA);
			if (rc == NEBC7_OK && cudaMalloc((void**)&S.dTable, sizeof(TexDesc) * S.table.size()) != cudaSuccess)
				rc = SetError(NEBC7_ENOMEM);
			if (rc == NEBC7_OK && cudaMemcpy(S.dTable, S.table.data(), sizeof(TexDesc) * S.table.size(), cudaMemcpyHostToDevice) != cudaSuccess)
				rc = SetError(NEBC7_ECUDA);
		}
		if (rc == NEBC7_OK && cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) != cudaSuccess)
			rc = SetError(NEBC7_ECUDA);
		for (size_t i = 0; i < ng && rc == NEBC7_OK; i++)
		{
			cudaEvent_t e;
			if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
				rc = SetError(NEBC7_ECUDA);
			else
				b->ev.push_back(e);
			if (rc == NEBC7_OK && i > 0)
			{
				cudaStream_t s2;
				if (cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking) != cudaSuccess)
					rc = SetError(NEBC7_ECUDA);
				else
					b->side.push_back(s2);
			}
		}
	}
	if (rc != NEBC7_OK)
	{
		FreeBatch(b);
		return rc;
	}
	/* without tuning: one launch per preset group when the batch mixes presets */
	b->chosen = b->sched[1].groups.size() > 1 ? 1 : 0;
	*out = b;
	return NEBC7_OK;
}

int nebc7_batch_tune(nebc7_batch* b, int trials, float* ms_out)
{
	if (!b || trials <= 0)
		return SetError(NEBC7_EINVAL);
	CK(cudaSetDevice(b->device));
	/* the trials rewrite the outputs: keep the starting blocks unless every
	   launch starts from scratch anyway */
	std::vector<uint8_t*> saved;
	int rc = NEBC7_OK;
	if (!b->fromScratch)
	{
		for (const nebc7_texture& t : b->tex)
		{
			const size_t bytes = size_t(t.w / 4) * (t.h / 4) * 16;
			uint8_t* p = nullptr;
			if (cudaMalloc((void**)&p, bytes) != cudaSuccess || cudaMemcpy(p, t.d_dst, bytes, cudaMemcpyDeviceToDevice) != cudaSuccess)
			{
				cudaFree(p);
				rc = SetError(NEBC7_ENOMEM);
				break;
			}
			saved.push_back(p);
		}
	}
	auto restore = [&]() {
		for (size_t i = 0; i < saved.size(); i++)
		{
			const nebc7_texture& t = b->tex[i];
			cudaMemcpyAsync(t.d_dst, saved[i], size_t(t.w / 4) * (t.h / 4) * 16, cudaMemcpyDeviceToDevice, b->cap);
		}
	};
	float best[2] = { 3.4e38f, 3.4e38f };
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	if (rc == NEBC7_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
		rc = SetError(NEBC7_ECUDA);
	/* best of `trials` replays of one plan's graph */
	auto measure = [&](int schedule, int staged, int ctas, float* out) -> int {
		if (int e = ApplyPlan(b, schedule, staged, ctas))
			return e;
		float m = 3.4e38f;
		for (int trial = 0; trial < trials; trial++)
		{
			cudaGraphExec_t g = nullptr;
			if (int e = GraphFor(b, schedule, &g))
				return e;
			restore();
			if (cudaEventRecord(e0, b->cap) != cudaSuccess || cudaGraphLaunch(g, b->cap) != cudaSuccess ||
				cudaEventRecord(e1, b->cap) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
				return SetError(NEBC7_ECUDA);
			float ms = 0;
			cudaEventElapsedTime(&ms, e0, e1);
			m = std::min(m, ms);
		}
		b->trials.push_back(nebc7_batch::Trial{ schedule, staged, ctas, m });
		best[schedule] = std::min(best[schedule], m);
		*out = m;
		return NEBC7_OK;
	};
	/* coordinate search from one mixed launch in the staged form at full
	   occupancy: the schedule, then the staged form, then fewer CTAs per SM,
	   each kept when it is faster */
	b->trials.clear();
	bool anyStaged = false;
	for (const BatchSchedule& S : b->sched)
		for (const BatchGroup& g : S.groups)
			anyStaged |= g.stagedOff >= 0;
	int cur[3] = { 0, 1, 0 };
	float curMs = 0;
	if (rc == NEBC7_OK)
		rc = measure(cur[0], cur[1], cur[2], &curMs);
	auto tryPlan = [&](int schedule, int staged, int ctas) {
		if (rc != NEBC7_OK)
			return;
		float m = 0;
		rc = measure(schedule, staged, ctas, &m);
		if (rc == NEBC7_OK && m < curMs)
		{
			cur[0] = schedule;
			cur[1] = staged;
			cur[2] = ctas;
			curMs = m;
		}
	};
	if (b->sched[1].groups.size() >= 2)
		tryPlan(1, cur[1], cur[2]);
	if (anyStaged)
		tryPlan(cur[0], 0, cur[2]);
	tryPlan(cur[0], cur[1], 2);
	if (rc == NEBC7_OK)
	{
		rc = ApplyPlan(b, cur[0], cur[1], cur[2]);
		if (ms_out)
		{
			ms_out[0] = best[0];
			ms_out[1] = best[1];
		}
	}
	restore();
	cudaStreamSynchronize(b->cap);
	for (uint8_t* p : saved)
		cudaFree(p);
	if (e0)
		cudaEventDestroy(e0);
	if (e1)
		cudaEventDestroy(e1);
	return rc;
}

int nebc7_batch_launch(nebc7_batch* b, void* stream)
{
	if (!b)
		return SetError(NEBC7_EINVAL);
	cudaGraphExec_t g = nullptr;
	if (int rc = GraphFor(b, b->chosen, &g))
		return rc;
	CK(cudaGraphLaunch(g, (cudaStream_t)stream));
	return NEBC7_OK;
}

int nebc7_batch_sums(nebc7_batch* b, void* stream, int64_t* errs, double* ssim)
{
	if (!b)
		return SetError(NEBC7_EINVAL);
	const size_t n = b->tex.size();
	const cudaStream_t st = (cudaStream_t)stream;
	if (errs)
		CK(cudaMemcpyAsync(errs, b->errs, sizeof(long long) * 2 * n, cudaMemcpyDeviceToHost, st));
	if (ssim)
		CK(cudaMemcpyAsync(ssim, b->ssims, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	return NEBC7_OK;
}

int nebc7_batch_set_schedule(nebc7_batch* b, int schedule)
{
	if (!b || schedule < 0 || schedule > 1)
		return SetError(NEBC7_EINVAL);
	b->chosen = schedule;
	return NEBC7_OK;
}

int nebc7_batch_plan(const nebc7_batch* b, int* schedule, int* staged, int* ctas_per_sm)
{
	if (!b)
		return SetError(NEBC7_EINVAL);
	if (schedule)
		*schedule = b->chosen;
	if (staged)
		*staged = b->staged;
	if (ctas_per_sm)
		*ctas_per_sm = b->ctasPerSm;
	return NEBC7_OK;
}

int nebc7_batch_set_plan(nebc7_batch* b, int schedule, int staged, int ctas_per_sm)
{
	if (!b || schedule < 0 || schedule > 1 || staged < 0 || staged > 1 || ctas_per_sm < 0 || ctas_per_sm > 64)
		return SetError(NEBC7_EINVAL);
	CK(cudaSetDevice(b->device));
	return ApplyPlan(b, schedule, staged, ctas_per_sm);
}

int nebc7_batch_trials(const nebc7_batch* b, int* schedule, int* staged, int* ctas_per_sm, float* ms, int cap)
{
	if (!b || cap < 0)
		return SetError(NEBC7_EINVAL);
	const int n = int(b->trials.size());
	for (int i = 0; i < n && i < cap; i++)
	{
		const nebc7_batch::Trial& t = b->trials[i];
		if (schedule)
			schedule[i] = t.schedule;
		if (staged)
			staged[i] = t.staged;
		if (ctas_per_sm)
			ctas_per_sm[i] = t.ctasPerSm;
		if (ms)
			ms[i] = t.ms;
	}
	return n;
}

int nebc7_batch_info(const nebc7_batch* b, int* schedule, int* launches, int* blocks)
{
	if (!b)
		return SetError(NEBC7_EINVAL);
	if (schedule)
		*schedule = b->chosen;
	if (launches)
	{
		/* per group: the block order (2), the encode (the staged form: the
		   first kernel, then a list and a kernel per stage), the sums */
		int n = 0;
		for (const BatchGroup& g : b->sched[b->chosen].groups)
			n += 2 + ((b->staged && g.stagedOff >= 0) ? 1 + 2 * kNumStages : 1) + 1;
		*launches = n;
	}
	if (blocks)
		*blocks = b->totalBlocks;
	return NEBC7_OK;
}

void nebc7_batch_destroy(nebc7_batch* b)
{
	FreeBatch(b);
}

int nebc7_server_create(const nebc7_server_config* cfg, nebc7_server** out)
{
	if (!cfg || !out || cfg->hbm_budget < 4096 || cfg->max_batch <= 0 || cfg->max_batch > 4096 || cfg->streams <= 0 ||
		cfg->streams > 64)
		return SetError(NEBC7_EINVAL);
	*out = nullptr;
	nebc7_server* sv = new nebc7_server;
	sv->cfg = *cfg;
	sv->t0 = NowSeconds();
	int rc = NEBC7_OK;
	if (cudaGetDevice(&sv->device) != cudaSuccess)
		rc = SetError(NEBC7_ECUDA);
	for (int d = 0; d < 2 && rc == NEBC7_OK; d++)
		rc = BuildTables(sv->device, d, &sv->T[d]);
	if (rc == NEBC7_OK && cudaMalloc((void**)&sv->arena, cfg->hbm_budget) != cudaSuccess)
		rc = SetError(NEBC7_ENOMEM);
	sv->alloc.Init(cfg->hbm_budget);
	sv->slots.resize(cfg->streams);
	const int cap = cfg->max_batch;
	for (ServerSlot& slot : sv->slots)
	{
		if (rc != NEBC7_OK)
			break;
		slot.copied.assign(cap, nullptr);
		for (cudaEvent_t& e : slot.copied)
			if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
				rc = SetError(NEBC7_ECUDA);
		if (rc == NEBC7_OK && (cudaHostAlloc((void**)&slot.hFlags, sizeof(int) * cap, cudaHostAllocMapped) != cudaSuccess ||
			cudaHostGetDevicePointer((void**)&slot.dFlags, slot.hFlags, 0) != cudaSuccess ||
			cudaMallocHost((void**)&slot.hRemaining, sizeof(int) * cap) != cudaSuccess ||
			cudaMalloc((void**)&slot.dRemaining, sizeof(int) * cap) != cudaSuccess ||
			cudaStreamCreateWithFlags(&slot.copies, cudaStreamNonBlocking) != cudaSuccess))
			rc = SetError(NEBC7_ENOMEM);
		if (rc != NEBC7_OK)
			break;
		if (cudaStreamCreateWithFlags(&slot.stream, cudaStreamNonBlocking) != cudaSuccess ||
			cudaEventCreateWithFlags(&slot.done, cudaEventDisableTiming) != cudaSuccess ||
			cudaMallocHost((void**)&slot.hTable, sizeof(TexDesc) * cap) != cudaSuccess ||
			cudaMallocHost((void**)&slot.hSums, sizeof(long long) * 4 * cap) != cudaSuccess ||
			cudaMalloc((void**)&slot.dTable, sizeof(TexDesc) * cap) != cudaSuccess ||
			cudaMalloc((void**)&slot.dSums, sizeof(long long) * 4 * cap) != cudaSuccess ||
			cudaMalloc((void**)&slot.dCounter, 256) != cudaSuccess)
			rc = SetError(NEBC7_ENOMEM);
		/* the staged form's records: a launch holds at most one block per
		   kServerBlockBytes of the arena */
		slot.stagedCap = int(std::min<size_t>(kServerStagedBlocks, cfg->hbm_budget / kServerBlockBytes + 1));
		if (rc == NEBC7_OK && cudaMalloc((void**)&slot.staged, StagedScratchBytes(slot.stagedCap)) != cudaSuccess)
			rc = SetError(NEBC7_ENOMEM);
	}
	/* size the mixed kernel's launch before any request arrives */
	if (rc == NEBC7_OK && GridForSlot(1, kVariantMixed) <= 0)
		rc = SetError(NEBC7_ECUDA);
	if (rc != NEBC7_OK)
	{
		FreeServer(sv);
		return rc;
	}
	sv->worker = std::thread(ServerLoop, sv);
	*out = sv;
	return NEBC7_OK;
}

int nebc7_server_submit(nebc7_server* sv, const uint8_t* bgra, const uint8_t* mask, long long stride, int w, int h,
	const nebc7_settings* settings, uint8_t* dst, int64_t* ticket)
{
	if (!sv || !ticket || !bgra || !dst)
		return SetError(NEBC7_EINVAL);
	if (int e = ValidateSettings(settings))
		return SetError(e);
	if (w <= 0 || h <= 0 || (w & 3) || (h & 3) || stride < (long long)w * 4)
		return SetError(NEBC7_EINVAL);
	if ((long long)(w / 4) * (h / 4) > 0x7FFFFFFF)
		return SetError(NEBC7_ETOOBIG);
	ServerRequest r;
	r.bgra = bgra;
	r.mask = mask;
	r.stride = stride;
	r.w = w;
	r.h = h;
	r.settings = *settings;
	r.dst = dst;
	r.bytes = RequestBytes(r);
	if (r.bytes > sv->cfg.hbm_budget)
		return SetError(NEBC7_ETOOBIG);
	r.tSubmit = NowSeconds();
	{
		std::lock_guard<std::mutex> lock(sv->mu);
		if (sv->stop)
			return SetError(NEBC7_EINVAL);
		const int64_t id = sv->nextId++;
		sv->reqs.emplace(id, r);
		sv->queued.push_back(id);
		*ticket = id;
	}
	sv->work.notify_one();
	return NEBC7_OK;
}

int nebc7_server_wait(nebc7_server* sv, int64_t ticket, double timeout_s, nebc7_request_info* info)
{
	if (!sv)
		return SetError(NEBC7_EINVAL);
	std::unique_lock<std::mutex> lock(sv->mu);
	auto it = sv->reqs.find(ticket);
	if (it == sv->reqs.end())
		return SetError(NEBC7_EINVAL);
	/* elements of the map keep their address while others are inserted */
	const ServerRequest* rp = &it->second;
	const auto done = [&] { return rp->state == 3 || rp->state < 0; };
	if (timeout_s < 0)
		sv->cv.wait(lock, done);
	else if (!sv->cv.wait_for(lock, std::chrono::duration<double>(timeout_s), done))
		return NEBC7_ELIMIT;
	const ServerRequest& r = *rp;
	const int rc = r.state < 0 ? -r.state : NEBC7_OK;
	if (info)
	{
		info->status = rc;
		info->queue_ms = (r.tLaunch - r.tSubmit) * 1e3;
		info->latency_ms = (r.tDone - r.tSubmit) * 1e3;
		info->submit_at_ms = (r.tSubmit - sv->t0) * 1e3;
		info->launch_at_ms = (r.tLaunch - sv->t0) * 1e3;
		info->done_at_ms = (r.tDone - sv->t0) * 1e3;
		info->slot = r.slot;
		info->launch = r.launch;
		info->errs[0] = r.errs[0];
		info->errs[1] = r.errs[1];
		info->ssim[0] = r.ssim[0];
		info->ssim[1] = r.ssim[1];
	}
	sv->reqs.erase(ticket);
	return rc;
}

int nebc7_server_stats(nebc7_server* sv, nebc7_server_counters* out)
{
	if (!sv || !out)
		return SetError(NEBC7_EINVAL);
	std::lock_guard<std::mutex> lock(sv->mu);
	out->completed = sv->completed;
	out->failed = sv->failed;
	out->launches = sv->launches;
	out->queued = (long long)sv->queued.size();
	out->bytes_in_use = (long long)sv->alloc.inUse;
	out->peak_bytes = (long long)sv->alloc.peak;
	return NEBC7_OK;
}

void nebc7_server_destroy(nebc7_server* sv)
{
	if (!sv)
		return;
	{
		std::lock_guard<std::mutex> lock(sv->mu);
		sv->stop = true;
	}
	sv->work.notify_all();
	if (sv->worker.joinable())
		sv->worker.join();
	FreeServer(sv);
}

int nebc7_prepare_device(const uint8_t* d_src, long long src_stride, int w, int h, uint8_t* d_padded, uint8_t* d_mask,
	int radius, void* stream)
{
	if (!d_src || !d_padded || w <= 0 || h <= 0 || src_stride < (long long)w * 4 || (src_stride & 3) ||
		((uintptr_t)d_src & 3) || ((uintptr_t)d_padded & 3) || ((uintptr_t)d_mask & 3))
		return SetError(NEBC7_EINVAL);
	const int pw = (std::max(4, w) + 3) & ~3, ph = (std::max(4, h) + 3) & ~3;
	if (std::max(pw, ph) > 16384)
		return SetError(NEBC7_ETOOBIG);
	const cudaStream_t st = (cudaStream_t)stream;
	const dim3 grid((pw + 255) / 256, ph);
	KPadTexture<<<grid, 256, 0, st>>>(d_src, src_stride, w, h, d_padded, (long long)pw * 4, pw, ph);
	CK(cudaGetLastError());
	if (d_mask)
	{
		KOutlineMask<<<grid, 256, 0, st>>>(d_padded, (long long)pw * 4, pw, ph, radius, d_mask);
		CK(cudaGetLastError());
	}
	return NEBC7_OK;
}

int nebc7_bad_blocks_device(const uint8_t* d_src, const uint8_t* d_decoded, const uint8_t* d_mask, long long stride, int w, int h,
	int linear, uint8_t* d_out, void* stream)
{
	if (!d_src || !d_decoded || !d_out || w <= 0 || h <= 0 || (w & 3) || (h & 3) || stride < (long long)w * 4 || (stride & 3) ||
		((uintptr_t)d_src & 3) || ((uintptr_t)d_decoded & 3) || ((uintptr_t)d_mask & 3) || ((uintptr_t)d_out & 3))
		return SetError(NEBC7_EINVAL);
	const dim3 grid((w / 4 + 1) / 2, h / 4);
	KBadBlocks<<<grid, 32, 0, (cudaStream_t)stream>>>(d_src, d_decoded, d_mask, stride, w, h, linear, d_out);
	CK(cudaGetLastError());
	return NEBC7_OK;
}

int nebc7_partition_map_device(const uint8_t* d_blocks, uint8_t* d_out, int nblocks, void* stream)
{
	if (!d_blocks || !d_out || nblocks < 0 || ((uintptr_t)d_blocks & 15) || ((uintptr_t)d_out & 15))
		return SetError(NEBC7_EINVAL);
	if (nblocks == 0)
		return NEBC7_OK;
	KPartitionMap<<<(nblocks + 255) / 256, 256, 0, (cudaStream_t)stream>>>(d_blocks, d_out, nblocks);
	CK(cudaGetLastError());
	return NEBC7_OK;
}

int nebc7_ktx_header(int w, int h, int flip, uint8_t* out)
{
	if (!out || w <= 0 || h <= 0 || std::max(w, h) > 16384)
		return SetError(NEBC7_EINVAL);
	const int pw = (std::max(4, w) + 3) & ~3, ph = (std::max(4, h) + 3) & ~3;
	/* KTX 1.1: identifier, endianness, GL format fields (BPTC RGBA, base
	   RGBA), image size in pixels, one face / level, an orientation
	   key/value ("KTXOrientation": "S=r,T=u" flipped, "S=r,T=d" otherwise),
	   then the level's
	   byte count: the layout the reference writes (src/Bc7Compress.cpp:439-463) */
	const uint32_t head[24] = {
		0x58544BABu, 0xBB313120u, 0x0A1A0A0Du, 0x04030201u,
		0, 1, 0, 0x8E8C, 0x1908,
		uint32_t(w), uint32_t(h), 0, 0, 1, 1,
		0x1C, 0x17, 0x4F58544Bu, 0x6E656972u, 0x69746174u, 0x53006E6Fu, 0x542C723Du, flip ? 0x00753Du : 0x00643Du,
		uint32_t(pw) * uint32_t(ph),
	};
	for (int i = 0; i < 24; i++)
		for (int b = 0; b < 4; b++)
			out[4 * i + b] = uint8_t(head[i] >> (8 * b));
	return NEBC7_OK;
}

int nebc7_launch_shape(int* ctas_per_sm, int* warps_per_cta, int* sm_count)
{
	int dev = 0, sms = 0, perSm = 0;
	CK(cudaGetDevice(&dev));
	CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	const nebc7_settings def = { 1, 9, 1, 1, 0, 0 };
	CK(kVariants[VariantSlot(def)].occupancy(&perSm));
	if (ctas_per_sm)
		*ctas_per_sm = perSm;
	if (warps_per_cta)
		*warps_per_cta = kWarpsPerCta;
	if (sm_count)
		*sm_count = sms;
	return NEBC7_OK;
}

} // extern "C"
