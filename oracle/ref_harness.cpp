/*
 * Harness around the reference encoder built from its own sources (test
 * infrastructure only; see ref_shim.h).  It supplies what the reference
 * leaves to its Windows build -- image IO (src/IO.h:7-11) and the job pool
 * (src/Worker.cpp:249 ProcessTexture, which needs boost outside Win32) --
 * and exports a small C API used by the fixture generator and the oracle
 * pinning tests:
 *
 *   nebc7_ref_encode_image      runs the reference CLI driver
 *                               Bc7MainWithArgs (src/Bc7Compress.cpp:267) on
 *                               an in-memory image with CLI flags, so padding
 *                               (:397-426), the alpha outline mask (:33-105)
 *                               and flag parsing (:284-378) are the
 *                               reference's own;
 *   nebc7_ref_compress_blocks   runs IBc7Core::pCompress
 *                               (src/Bc7Core.cpp:1936) on independent 4x4
 *                               cells with caller masks;
 *   nebc7_ref_decompress_blocks runs IBc7Core::pDecompress (:1904).
 *
 * Jobs are dealt in 256-block units like src/Worker.cpp:25-57, and the
 * per-job error / SSIM partial sums are reduced in job order so that the
 * double sums are reproducible.
 */
#include "ref_shim.h"

#include "Bc7Core.h"
#include "Worker.h"

#include <atomic>
#include <string>
#include <thread>
#include <vector>

int gNebc7RefQuiet = 1;
std::atomic<int> gNebc7RefSelfCheckFailures{0};

bool GetBc7Core(void* bc7Core);
int Bc7MainWithArgs(const IBc7Core& bc7Core, const std::vector<std::string>& args);

namespace {

struct MemoryImage
{
	const uint8_t* bgra = nullptr;
	int w = 0, h = 0;
	const uint8_t* preload = nullptr;  // existing BC7 payload, or null
	uint8_t* out = nullptr;            // captured BC7 payload
	int out_size = 0;
	int threads = 1;
	int64_t err_alpha = 0, err_color = 0;
	double ssim_alpha = 0, ssim_color = 0;
	bool saved = false;
};

MemoryImage gImage;

int gThreads = 1;

struct JobSums
{
	int64_t a = 0, c = 0;
	BlockSSIM s = BlockSSIM(0, 0);
};

void RunJobs(const std::vector<WorkerItem>& items, int stride, PBlockKernel kernel, int threads, int64_t& errA, int64_t& errC, BlockSSIM& ssim)
{
	const size_t job = 0x100;
	const size_t njobs = (items.size() + job - 1) / job;
	std::vector<JobSums> sums(njobs);
	std::atomic<size_t> next{0};

	auto proc = [&]() {
		for (;;)
		{
			size_t j = next.fetch_add(1);
			if (j >= njobs)
				break;
			size_t b = j * job;
			size_t e = b + job < items.size() ? b + job : items.size();
			kernel(items.data() + b, items.data() + e, stride, sums[j].a, sums[j].c, sums[j].s);
		}
	};

	if (threads <= 1)
	{
		proc();
	}
	else
	{
		std::vector<std::thread> pool;
		for (int t = 0; t < threads; t++)
			pool.emplace_back(proc);
		for (auto& t : pool)
			t.join();
	}

	errA = 0;
	errC = 0;
	ssim = BlockSSIM(0, 0);
	for (const auto& s : sums)
	{
		errA += s.a;
		errC += s.c;
		ssim.Alpha += s.s.Alpha;
		ssim.Color += s.s.Color;
	}
}

} // namespace

/* src/Worker.h:6 -- the reference's texture job splitter (src/Worker.cpp:249-280). */
void ProcessTexture(uint8_t* dst, uint8_t* src_bgra, uint8_t* mask_agrb, int stride, int src_w, int src_h, PBlockKernel blockKernel, size_t block_size, int64_t& pErrorAlpha, int64_t& pErrorColor, BlockSSIM& pssim)
{
	std::vector<WorkerItem> items;
	items.reserve(size_t(src_w / 4) * size_t(src_h / 4));

	uint8_t* output = dst;
	for (int y = 0; y < src_h; y += 4)
	{
		uint8_t* cell = src_bgra + y * stride;
		uint8_t* mask = mask_agrb + y * stride;
		for (int x = 0; x < src_w; x += 4)
		{
			items.emplace_back(output, cell, mask);
			output += block_size;
			cell += 16;
			mask += 16;
		}
	}

	RunJobs(items, stride, blockKernel, gThreads, pErrorAlpha, pErrorColor, pssim);

	gImage.err_alpha = pErrorAlpha;
	gImage.err_color = pErrorColor;
	gImage.ssim_alpha = pssim.Alpha;
	gImage.ssim_color = pssim.Color;
}

bool ReadImage(const char* src_name, uint8_t*& pixels, int& width, int& height, bool flip)
{
	(void)src_name;
	(void)flip;  // in-memory images are already top-down
	if (!gImage.bgra)
		return false;
	width = gImage.w;
	height = gImage.h;
	pixels = new uint8_t[size_t(width) * size_t(height) * 4];
	memcpy(pixels, gImage.bgra, size_t(width) * size_t(height) * 4);
	return true;
}

void LoadBc7(const char* name, int position, uint8_t* buffer, int size)
{
	(void)name;
	(void)position;
	if (gImage.preload)
		memcpy(buffer, gImage.preload, size_t(size));
}

void SaveBc7(const char* name, const uint8_t* head, int position, const uint8_t* buffer, int size)
{
	(void)name;
	(void)head;
	(void)position;
	if (gImage.out && size <= gImage.out_size)
	{
		memcpy(gImage.out, buffer, size_t(size));
		gImage.saved = true;
	}
}

extern "C" {

int nebc7_ref_denoise() { return kDenoise; }
int nebc7_ref_denoise_step() { return kDenoiseStep; }
int nebc7_ref_selfcheck_failures() { return gNebc7RefSelfCheckFailures.load(); }

/*
 * Encodes a w x h BGRA image through the reference CLI driver.  `flags` is a
 * space-separated list of CLI switches ("/nomask /noflip", "/draft", "/slow",
 * "/data", "/retina").  `out` receives the padded texture's BC7 payload
 * (padded_w * padded_h bytes, padded sides rounded up to 4); `out_size` is
 * its capacity.  err[0..1] = alpha / color error sums and ssim[0..1] = SSIM
 * sums exactly as the CLI computes them.  Returns 0 on success.
 */
int nebc7_ref_encode_image(const uint8_t* bgra, int w, int h, const char* flags, const uint8_t* preload,
	uint8_t* out, int out_size, int threads, int64_t* err, double* ssim)
{
	gImage = MemoryImage();
	gImage.bgra = bgra;
	gImage.w = w;
	gImage.h = h;
	gImage.preload = preload;
	gImage.out = out;
	gImage.out_size = out_size;
	gThreads = threads > 0 ? threads : 1;

	std::vector<std::string> args;
	{
		std::string f = flags ? flags : "";
		size_t p = 0;
		while (p < f.size())
		{
			size_t q = f.find(' ', p);
			if (q == std::string::npos)
				q = f.size();
			if (q > p)
				args.emplace_back(f.substr(p, q - p));
			p = q + 1;
		}
	}
	args.emplace_back("memory.png");
	args.emplace_back("memory.ktx");

	IBc7Core core{};
	if (!GetBc7Core(&core))
		return 2;

	int rc = Bc7MainWithArgs(core, args);
	if (rc != 0)
		return rc;
	if (!gImage.saved)
		return 3;

	if (err)
	{
		err[0] = gImage.err_alpha;
		err[1] = gImage.err_color;
	}
	if (ssim)
	{
		ssim[0] = gImage.ssim_alpha;
		ssim[1] = gImage.ssim_color;
	}
	return 0;
}

/*
 * Compresses n independent cells.  cells / masks hold 64 bytes per block
 * (4 rows of 4 BGRA pixels; mask bytes in A,G,R,B order, 0x00 or 0xFF);
 * io holds 16 bytes per block, read as the starting block and overwritten.
 */
int nebc7_ref_compress_blocks(const uint8_t* cells, const uint8_t* masks, uint8_t* io, int n,
	int doDraft, int doNormal, int doSlow, int linearData, int threads, int64_t* err, double* ssim)
{
	IBc7Core core{};
	if (!GetBc7Core(&core))
		return 2;
	core.pInitTables(doDraft != 0, doNormal != 0, doSlow != 0, linearData != 0);

	std::vector<WorkerItem> items;
	items.reserve(size_t(n));
	for (int i = 0; i < n; i++)
	{
		items.emplace_back(io + size_t(i) * 16, const_cast<uint8_t*>(cells) + size_t(i) * 64, const_cast<uint8_t*>(masks) + size_t(i) * 64);
	}

	int64_t a = 0, c = 0;
	BlockSSIM s(0, 0);
	RunJobs(items, 16, core.pCompress, threads, a, c, s);
	if (err)
	{
		err[0] = a;
		err[1] = c;
	}
	if (ssim)
	{
		ssim[0] = s.Alpha;
		ssim[1] = s.Color;
	}
	return 0;
}

/* Decodes n blocks into 64 bytes of BGRA per block (4 rows of 4 pixels). */
int nebc7_ref_decompress_blocks(uint8_t* blocks, uint8_t* bgra, int n)
{
	IBc7Core core{};
	if (!GetBc7Core(&core))
		return 2;
	std::vector<WorkerItem> items;
	items.reserve(size_t(n));
	for (int i = 0; i < n; i++)
	{
		items.emplace_back(blocks + size_t(i) * 16, bgra + size_t(i) * 64, nullptr);
	}
	int64_t a = 0, c = 0;
	BlockSSIM s(0, 0);
	RunJobs(items, 16, core.pDecompress, 1, a, c, s);
	return 0;
}

} // extern "C"

/* Table access for pinning the port's table generation (src/Bc7Tables.h). */
extern uint8_t gTableDeltas2_Value8[0x100][0x100 * 0x100];
extern uint8_t gTableDeltas2_Value7[0x100][0x80 * 0x80];
extern uint8_t gTableDeltas2_Value6[0x100][0x40 * 0x40];
extern uint8_t gTableDeltas2_Value5[0x100][0x20 * 0x20];
extern uint16_t gTableCuts2_Value8[0x100][0x100];
extern uint16_t gTableCuts2_Value6[0x100][0x40];
extern uint16_t gTableCuts2_Value5[0x100][0x20];
extern uint8_t gTableDeltas3_Value7Shared[0x100][0x80 * 0x80];
extern uint8_t gTableDeltas3_Value6[0x100][0x40 * 0x40];
extern uint8_t gTableDeltas3_Value5[0x100][0x20 * 0x20];
extern uint16_t gTableCuts3_Value7Shared[0x100][0x80];
extern uint16_t gTableCuts3_Value5[0x100][0x20];
extern uint8_t gTableDeltas4Half_Value8[0x100][0x100 * 0x80];
extern uint8_t gTableDeltas2Half_Value8[0x100][0x100 * 0x80];

extern "C" const void* nebc7_ref_table(int id, int* size)
{
	const void* p = nullptr;
	int s = 0;
	switch (id)
	{
	case 0: p = gTableDeltas2_Value8; s = sizeof(gTableDeltas2_Value8); break;
	case 1: p = gTableDeltas2_Value7; s = sizeof(gTableDeltas2_Value7); break;
	case 2: p = gTableDeltas2_Value6; s = sizeof(gTableDeltas2_Value6); break;
	case 3: p = gTableDeltas2_Value5; s = sizeof(gTableDeltas2_Value5); break;
	case 4: p = gTableCuts2_Value8; s = sizeof(gTableCuts2_Value8); break;
	case 5: p = gTableCuts2_Value6; s = sizeof(gTableCuts2_Value6); break;
	case 6: p = gTableCuts2_Value5; s = sizeof(gTableCuts2_Value5); break;
	case 7: p = gTableDeltas3_Value7Shared; s = sizeof(gTableDeltas3_Value7Shared); break;
	case 8: p = gTableDeltas3_Value6; s = sizeof(gTableDeltas3_Value6); break;
	case 9: p = gTableDeltas3_Value5; s = sizeof(gTableDeltas3_Value5); break;
	case 10: p = gTableCuts3_Value7Shared; s = sizeof(gTableCuts3_Value7Shared); break;
	case 11: p = gTableCuts3_Value5; s = sizeof(gTableCuts3_Value5); break;
	case 12: p = gTableDeltas4Half_Value8; s = sizeof(gTableDeltas4Half_Value8); break;
	case 13: p = gTableDeltas2Half_Value8; s = sizeof(gTableDeltas2Half_Value8); break;
	}
	if (size)
		*size = s;
	return p;
}
