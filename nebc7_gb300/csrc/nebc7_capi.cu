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

#include "../../include/nebc7_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string.h>
#include <vector>

using namespace nebc7;

namespace {

constexpr int kMaxDevices = 16;

struct DeviceTables
{
	bool built = false;
	LevelTables t{};
	void* mem[14] = {};
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

int BuildTables(int dev, int denoise, const LevelTables** out)
{
	std::lock_guard<std::mutex> lock(gMutex);
	if (dev < 0 || dev >= kMaxDevices)
		return SetError(NEBC7_EINVAL);
	DeviceTables& D = gTables[dev][denoise];
	if (!D.built)
	{
		const size_t sizes[23] = {
			size_t(256) * 65536, size_t(256) * 16384, size_t(256) * 4096, size_t(256) * 1024,
			size_t(256) * 256 * 2, size_t(256) * 64 * 2, size_t(256) * 32 * 2,
			size_t(256) * 16384, size_t(256) * 4096, size_t(256) * 1024,
			size_t(256) * 128 * 2, size_t(256) * 32 * 2,
			size_t(256) * 32768, size_t(256) * 32768,
		};
		for (int i = 0; i < 14; i++)
		{
			if (cudaMalloc(&D.mem[i], sizes[i]) != cudaSuccess)
			{
				for (int j = 0; j < i; j++)
					cudaFree(D.mem[j]);
				return SetError(NEBC7_ENOMEM);
			}
		}
		uint8_t* d3v8 = nullptr;
		if (cudaMalloc(&d3v8, size_t(256) * 65536) != cudaSuccess)
			return SetError(NEBC7_ENOMEM);
		uint8_t* d2v8 = (uint8_t*)D.mem[0];
		const int tb = 256;
		auto grid = [&](uint64_t n) { return unsigned((n + tb - 1) / tb); };
		/* 3-bit index tables (reference src/Bc7Tables.cpp:587-641) */
		KBuildFull<<<grid(uint64_t(256) * 65536), tb>>>(d3v8, 8, denoise, 0);
		KReduce<<<grid(uint64_t(256) * 16384), tb>>>(d3v8, (uint8_t*)D.mem[7], 7, 1);
		KReduce<<<grid(uint64_t(256) * 4096), tb>>>(d3v8, (uint8_t*)D.mem[8], 6, 0);
		KReduce<<<grid(uint64_t(256) * 1024), tb>>>(d3v8, (uint8_t*)D.mem[9], 5, 0);
		KCut<<<grid(256 * 128), tb>>>((uint8_t*)D.mem[7], (uint16_t*)D.mem[10], 7);
		KCut<<<grid(256 * 32), tb>>>((uint8_t*)D.mem[9], (uint16_t*)D.mem[11], 5);
		/* 2-bit index tables (:643-692) */
		KBuildFull<<<grid(uint64_t(256) * 65536), tb>>>(d2v8, 4, denoise, 0);
		KReduce<<<grid(uint64_t(256) * 16384), tb>>>(d2v8, (uint8_t*)D.mem[1], 7, 0);
		KReduce<<<grid(uint64_t(256) * 4096), tb>>>(d2v8, (uint8_t*)D.mem[2], 6, 0);
		KReduce<<<grid(uint64_t(256) * 1024), tb>>>(d2v8, (uint8_t*)D.mem[3], 5, 0);
		KCut<<<grid(256 * 256), tb>>>(d2v8, (uint16_t*)D.mem[4], 8);
		KCut<<<grid(256 * 64), tb>>>((uint8_t*)D.mem[2], (uint16_t*)D.mem[5], 6);
		KCut<<<grid(256 * 32), tb>>>((uint8_t*)D.mem[3], (uint16_t*)D.mem[6], 5);
		/* 4-bit and 2-of-4-bit nibble tables (:694-776) */
		KBuildFull<<<grid(uint64_t(256) * 32768), tb>>>((uint8_t*)D.mem[12], 16, denoise, 1);
		KHalfFrom2<<<grid(uint64_t(256) * 32768), tb>>>(d2v8, (uint8_t*)D.mem[13]);
		const cudaError_t e = cudaDeviceSynchronize();
		cudaFree(d3v8);
		if (e != cudaSuccess)
			return SetError(NEBC7_ECUDA);
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
		D.built = true;
	}
	*out = &D.t;
	return NEBC7_OK;
}

Params MakeParams(const nebc7_settings& s)
{
	Params p;
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
	if (!s || (s->denoise != 0 && s->denoise != 1) || s->denoiseStep < 0 || s->denoiseStep > 4096)
		return NEBC7_EINVAL;
	if ((s->doNormal || s->doSlow) && !kHasNormalPasses)
		return NEBC7_EUNSUPPORTED;
	return NEBC7_OK;
}

/* The encode instantiations: denoise shift x passes x code shape. */
struct EncodeVariant
{
	cudaError_t (*launch)(int, cudaStream_t, const Job&, const LevelTables&, const LevelTables&);
	cudaError_t (*occupancy)(int*);
};

constexpr int kNumVariants = 6;
constexpr int kVariantMixed = 5;   /* batches: kDenoise per texture */
const EncodeVariant kVariants[kNumVariants] = {
	{ LaunchEncodeKernel<0, false, kShapeCompact>, EncodeKernelOccupancy<0, false, kShapeCompact> },
	{ LaunchEncodeKernel<0, true, kShapeOutlined>, EncodeKernelOccupancy<0, true, kShapeOutlined> },
	{ LaunchEncodeKernel<1, false, kShapeCompact>, EncodeKernelOccupancy<1, false, kShapeCompact> },
	{ LaunchEncodeKernel<1, true, kShapeCompact>, EncodeKernelOccupancy<1, true, kShapeCompact> },
	{ LaunchEncodeKernel<1, true, kShapeOutlined>, EncodeKernelOccupancy<1, true, kShapeOutlined> },
	{ LaunchEncodeKernel<kAnyDenoise, true, kShapeOutlined>, EncodeKernelOccupancy<kAnyDenoise, true, kShapeOutlined> },
};

/* Picks the instantiation: the compact shape for the stepped default preset
   (kDenoise 1, refinement without /slow or /data), the outlined one where
   the full searches dominate (measured on the 1024x1024 and 2048x2048
   workloads). */
int VariantSlot(const nebc7_settings& s)
{
	if (!s.doNormal)
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

int GridForSlot(int nblocks, int slot)
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
			L.perSm[slot] = n > 0 ? n : 1;
		}
		sms = L.sms;
		perSm = L.perSm[slot];
	}
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
	job.single.P = MakeParams(s);
	job.ntex = 1;
	job.total = nblocks;
	job.results = results;
	job.counter = counter;
	job.status = status;
	return job;
}

/* Scratch of one encode: the work-queue head and status word, the reduced
   sums and, when sums are wanted, one BlockResult per block. */
size_t EncodeScratchBytes(int nblocks, bool wantSums)
{
	return 256 + (wantSums ? size_t(nblocks) * sizeof(BlockResult) : 0) + 64;
}

/* Enqueues one encode.  `scratchIn` (EncodeScratchBytes bytes, 256-byte
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
	if (!scratch && cudaMallocAsync((void**)&scratch, EncodeScratchBytes(nblocks, wantSums), stream) != cudaSuccess)
		return SetError(NEBC7_ENOMEM);
	int* counter = (int*)scratch;
	int* status = counter + 1;
	long long* sums = (long long*)(scratch + 64);
	double* ssums = (double*)(scratch + 128);
	BlockResult* results = wantSums ? (BlockResult*)(scratch + 256) : nullptr;
	CK(cudaMemsetAsync(scratch, 0, 256, stream));

	const Job job = SingleJob(dst, bgra, mask, stride, blocksW, nblocks, s, results, counter, status);
	const int grid = GridFor(nblocks, s);
	if (grid <= 0)
	{
		if (!scratchIn)
			cudaFreeAsync(scratch, stream);
		return SetError(NEBC7_ECUDA);
	}
	CK(kVariants[VariantSlot(s)].launch(grid, stream, job, *T, *T));

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
	if (!s.doNormal)
		return 1.0;
	if (s.linearData)
		return 7200.0;
	if (s.doSlow)
		return 480.0;
	if (!s.denoise || s.denoiseStep == 0)
		return 400.0;
	return 11.0;
}

struct BatchGroup
{
	int slot;                 /* kernel instantiation */
	int firstTex, ntex;       /* entries of the schedule's texture table */
	int queueBase;            /* offset of its queue positions in the results */
	int total;                /* blocks */
	int grid;
};

struct BatchSchedule
{
	std::vector<TexDesc> table;      /* host copy, groups contiguous */
	std::vector<BatchGroup> groups;
	TexDesc* dTable = nullptr;       /* device copy */
	cudaGraphExec_t graph = nullptr;
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
	int* counters = nullptr;
	BlockResult* results = nullptr;
	long long* errs = nullptr;
	double* ssims = nullptr;
	cudaStream_t cap = nullptr;      /* capture stream */
	std::vector<cudaStream_t> side;  /* concurrent preset groups */
	std::vector<cudaEvent_t> ev;     /* fork / join */
	const LevelTables* T[2] = { nullptr, nullptr };
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
		d.P = MakeParams(t.settings);
		S.table.push_back(d);
		g.ntex++;
		g.total += d.nblocks;
		queue += d.nblocks;
	}
	for (BatchGroup& g : S.groups)
		g.grid = GridForSlot(g.total, g.slot);
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
		job.single = S.table[G.firstTex];
		const cudaStream_t gs = g == 0 ? st : b->side[g - 1];
		CK(kVariants[G.slot].launch(G.grid, gs, job, *b->T[0], *b->T[1]));
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
	delete b;
}

} // namespace

/* ---- allocation-free encode -------------------------------------------- */

/* Largest texture nebc7_encode_device_noalloc accepts: 65536 blocks
   (1024x1024 pixels).  Its scratch lives in this fixed device array instead
   of coming from an allocator: 256 bytes for the work-queue head and the
   status word, then one BlockResult per block for the error / SSIM sums. */
constexpr int kNoAllocMaxBlocks = 65536;
constexpr size_t kNoAllocScratchBytes = 256 + size_t(kNoAllocMaxBlocks) * sizeof(BlockResult);
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
	/* the queue head and status word must start at zero */
	CK(cudaMemsetAsync(scratch, 0, 256, st));
	const Job job = SingleJob(d_dst, d_bgra, d_mask, stride, w / 4, int(nb), *settings,
		d_sums ? (BlockResult*)(scratch + 256) : nullptr, (int*)scratch, (int*)scratch + 1);
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
	if (!ReserveSlot(slot, offScratch + EncodeScratchBytes(int(nb), true)))
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

int nebc7_init_device(int denoise)
{
	if (denoise != 0 && denoise != 1)
		return SetError(NEBC7_EINVAL);
	int dev = 0;
	CK(cudaGetDevice(&dev));
	const LevelTables* T = nullptr;
	return BuildTables(dev, denoise, &T);
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
		if (cudaMalloc((void**)&b->dmem, bytes) != cudaSuccess)
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
	for (int trial = 0; trial < trials && rc == NEBC7_OK; trial++)
	{
		for (int w = 0; w < 2 && rc == NEBC7_OK; w++)
		{
			if (w == 1 && b->sched[1].groups.size() < 2)
				continue;   /* same as the mixed launch */
			cudaGraphExec_t g = nullptr;
			rc = GraphFor(b, w, &g);
			if (rc != NEBC7_OK)
				break;
			restore();
			if (cudaEventRecord(e0, b->cap) != cudaSuccess || cudaGraphLaunch(g, b->cap) != cudaSuccess ||
				cudaEventRecord(e1, b->cap) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
			{
				rc = SetError(NEBC7_ECUDA);
				break;
			}
			float ms = 0;
			cudaEventElapsedTime(&ms, e0, e1);
			best[w] = std::min(best[w], ms);
		}
	}
	if (rc == NEBC7_OK)
	{
		b->chosen = best[1] < best[0] ? 1 : 0;
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

int nebc7_batch_info(const nebc7_batch* b, int* schedule, int* launches, int* blocks)
{
	if (!b)
		return SetError(NEBC7_EINVAL);
	if (schedule)
		*schedule = b->chosen;
	if (launches)
		*launches = int(b->sched[b->chosen].groups.size());
	if (blocks)
		*blocks = b->totalBlocks;
	return NEBC7_OK;
}

void nebc7_batch_destroy(nebc7_batch* b)
{
	FreeBatch(b);
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
