/*
 * CPU oracle for the BC7 block encoder -- C API (test infrastructure only;
 * see port_tables.h).  Mirrors the reference's block kernels
 * (src/Bc7Core.cpp:1904 DecompressKernel, :1936 CompressKernel) and the
 * texture front end of its CLI (src/Bc7Compress.cpp:20-105 masks,
 * :397-426 padding), dealing 256-block jobs to std::threads like
 * src/Worker.cpp.  Used by the parity tests as the checker and by
 * bench.py as the CPU baseline.
 */
#include "port_core.h"
#include "port_counters.h"

#include <atomic>
#include <string.h>
#include <thread>
#include <vector>

using namespace nebc7_oracle;

namespace {

struct JobSums
{
	int64_t a = 0, c = 0;
	double sa = 0, sc = 0;
};

/* Loads one block into a Cell the way CompressKernel does
   (src/Bc7Core.cpp:1942-1976): BGRA rows -> A,G,R,B; mask rows as given. */
void LoadCell(Cell& cell, const uint8_t* bgra, const uint8_t* mask, int stride)
{
	for (int y = 0; y < 4; y++)
		for (int x = 0; x < 4; x++)
		{
			const uint8_t* p = bgra + y * stride + x * 4;
			const uint8_t* m = mask + y * stride + x * 4;
			const int i = y * 4 + x;
			cell.img[i][0] = p[3];
			cell.img[i][1] = p[1];
			cell.img[i][2] = p[2];
			cell.img[i][3] = p[0];
			cell.msk[i][0] = m[0];
			cell.msk[i][1] = m[1];
			cell.msk[i][2] = m[2];
			cell.msk[i][3] = m[3];
		}
}

template<class F>
void ParallelJobs(int nblocks, int threads, F&& fn, JobSums& total)
{
	const int job = 0x100;
	const int njobs = (nblocks + job - 1) / job;
	std::vector<JobSums> sums(size_t(njobs > 0 ? njobs : 1));
	std::atomic<int> next{ 0 };
	auto proc = [&]() {
		Cell* cell = new Cell();
		for (;;)
		{
			const int j = next.fetch_add(1);
			if (j >= njobs)
				break;
			const int b = j * job;
			const int e = b + job < nblocks ? b + job : nblocks;
			for (int k = b; k < e; k++)
				fn(*cell, k, sums[size_t(j)]);
		}
		delete cell;
	};
	if (threads <= 1)
		proc();
	else
	{
		std::vector<std::thread> pool;
		for (int t = 0; t < threads; t++)
			pool.emplace_back(proc);
		for (auto& t : pool)
			t.join();
	}
	for (int j = 0; j < njobs; j++)
	{
		total.a += sums[size_t(j)].a;
		total.c += sums[size_t(j)].c;
		total.sa += sums[size_t(j)].sa;
		total.sc += sums[size_t(j)].sc;
	}
}

} // namespace

#ifdef NEBC7_PORT_COUNTERS
namespace nebc7_oracle {
std::atomic<uint64_t> gWork[kNumWorkCounters];
}
#endif

extern "C" {

/* OPTION_PCA for the encodes that follow (0 off, the default). */
void nebc7_oracle_set_pca(int on)
{
	SetPca(on != 0);
}

/* The work counters (port_counters.h) since the last reset, in WorkCounter
   order; returns how many there are (0 in the plain build). */
int nebc7_oracle_work(uint64_t* out, int reset)
{
#ifdef NEBC7_PORT_COUNTERS
	for (int i = 0; i < kNumWorkCounters; i++)
		out[i] = reset ? gWork[i].exchange(0) : gWork[i].load();
	return kNumWorkCounters;
#else
	(void)out;
	(void)reset;
	return 0;
#endif
}

/* Builds the level tables for one kDenoise value ahead of timing. */
void nebc7_oracle_init(int denoise)
{
	GetLevelTables(denoise);
	GetSelection();
}

/*
 * Compresses the blocks of a padded texture (w, h multiples of 4) in place:
 * dst holds w*h/16 blocks read as the starting encoding and overwritten.
 * bgra / mask: rows of w pixels, stride bytes apart.  err[0..1] and
 * ssim[0..1] receive the sums CompressKernel accumulates.
 */
int nebc7_oracle_compress_texture(uint8_t* dst, const uint8_t* bgra, const uint8_t* mask, int stride, int w, int h,
	int denoise, int denoiseStep, int doDraft, int doNormal, int doSlow, int linearData, int threads,
	int64_t* err, double* ssim)
{
	if (w <= 0 || h <= 0 || (w & 3) || (h & 3) || stride < w * 4)
		return 1;
	if (denoise < 0 || denoise > 1)
		return 1;
	Config cfg;
	MakeConfig(cfg, denoise, denoiseStep, doDraft != 0, doNormal != 0, doSlow != 0, linearData != 0);
	cfg.mode6Index2Only = doDraft == 2;   /* doDraft 2: the Mode6Index2-only draft chain */
	const int bw = w / 4;
	const int nblocks = bw * (h / 4);
	JobSums total;
	ParallelJobs(nblocks, threads, [&](Cell& cell, int k, JobSums& s) {
		const int bx = k % bw, by = k / bw;
		const size_t off = size_t(by) * 4 * size_t(stride) + size_t(bx) * 16;
		LoadCell(cell, bgra + off, mask + off, stride);
		CompressBlock(cfg, dst + size_t(k) * 16, cell);
		s.a += int64_t(cell.errAlpha) << (cfg.denoise + cfg.denoise);
		s.c += int64_t(cell.errTotal - cell.errAlpha) << (cfg.denoise + cfg.denoise);
		s.sa += cell.qualityAlpha;
		s.sc += cell.qualityColor;
	}, total);
	if (err)
	{
		err[0] = total.a;
		err[1] = total.c;
	}
	if (ssim)
	{
		ssim[0] = total.sa;
		ssim[1] = total.sc;
	}
	return 0;
}

/* Independent cells: 64 bytes of BGRA and 64 bytes of mask per block, io
   16 bytes per block (starting encoding in, result out). */
int nebc7_oracle_compress_blocks(const uint8_t* cells, const uint8_t* masks, uint8_t* io, int n,
	int denoise, int denoiseStep, int doDraft, int doNormal, int doSlow, int linearData, int threads,
	int64_t* err, double* ssim)
{
	if (n < 0 || denoise < 0 || denoise > 1)
		return 1;
	Config cfg;
	MakeConfig(cfg, denoise, denoiseStep, doDraft != 0, doNormal != 0, doSlow != 0, linearData != 0);
	cfg.mode6Index2Only = doDraft == 2;   /* doDraft 2: the Mode6Index2-only draft chain */
	JobSums total;
	ParallelJobs(n, threads, [&](Cell& cell, int k, JobSums& s) {
		LoadCell(cell, cells + size_t(k) * 64, masks + size_t(k) * 64, 16);
		CompressBlock(cfg, io + size_t(k) * 16, cell);
		s.a += int64_t(cell.errAlpha) << (cfg.denoise + cfg.denoise);
		s.c += int64_t(cell.errTotal - cell.errAlpha) << (cfg.denoise + cfg.denoise);
		s.sa += cell.qualityAlpha;
		s.sc += cell.qualityColor;
	}, total);
	if (err)
	{
		err[0] = total.a;
		err[1] = total.c;
	}
	if (ssim)
	{
		ssim[0] = total.sa;
		ssim[1] = total.sc;
	}
	return 0;
}

/* Decodes n blocks to 64 bytes of BGRA each (src/Bc7Core.cpp:1904). */
int nebc7_oracle_decompress_blocks(const uint8_t* blocks, uint8_t* bgra, int n)
{
	Cell* cell = new Cell();
	for (int k = 0; k < n; k++)
	{
		DecompressBlock(blocks + size_t(k) * 16, *cell);
		for (int i = 0; i < 16; i++)
		{
			uint8_t* p = bgra + size_t(k) * 64 + size_t(i) * 4;
			p[0] = cell->img[i][3];
			p[1] = cell->img[i][1];
			p[2] = cell->img[i][2];
			p[3] = cell->img[i][0];
		}
	}
	delete cell;
	return 0;
}

/*
 * The CLI's texture preparation (src/Bc7Compress.cpp:397-426 padding by
 * edge replication to multiples of 4, at least 4; :33-105 alpha mask with
 * an outline of `radius` pixels, radius < 0 meaning a full mask as with
 * /nomask or /data :20-31).  src: w x h BGRA; padded: pw x ph BGRA;
 * mask: pw x ph, 4 bytes per pixel in A,G,R,B order.
 */
int nebc7_oracle_prepare_texture(const uint8_t* src, int w, int h, uint8_t* padded, uint8_t* mask, int radius)
{
	if (w <= 0 || h <= 0)
		return 1;
	const int pw = ((w > 4 ? w : 4) + 3) & ~3;
	const int ph = ((h > 4 ? h : 4) + 3) & ~3;
	for (int y = 0; y < h; y++)
	{
		memcpy(padded + size_t(y) * pw * 4, src + size_t(y) * w * 4, size_t(w) * 4);
		for (int x = w; x < pw; x++)
			memcpy(padded + (size_t(y) * pw + x) * 4, src + (size_t(y) * w + w - 1) * 4, 4);
	}
	for (int y = h; y < ph; y++)
		memcpy(padded + size_t(y) * pw * 4, padded + size_t(h - 1) * pw * 4, size_t(pw) * 4);

	if (radius < 0)
	{
		memset(mask, 0xFF, size_t(pw) * ph * 4);
		return 0;
	}
	/* sliding (2r+1)^2 box count of non-zero alpha, as a running sum */
	std::vector<int> buf(size_t(radius + pw + radius + 15), 0);
	auto alphaOn = [&](int y, int x) { return padded[(size_t(y) * pw + x) * 4 + 3] != 0 ? 1 : 0; };
	for (int y = 0; y < radius && y < ph; y++)
		for (int i = 0; i < pw; i++)
			buf[size_t(radius + i)] += alphaOn(y, i);
	for (int y = 0; y < ph; y++)
	{
		if (y + radius < ph)
			for (int i = 0; i < pw; i++)
				buf[size_t(radius + i)] += alphaOn(y + radius, i);
		int sum = 0;
		for (int i = 0; i < radius + radius; i++)
			sum -= buf[size_t(i)];
		for (int i = 0; i < pw; i++)
		{
			sum -= buf[size_t(radius + radius + i)];
			const uint8_t v = (sum < 0) ? 0xFF : 0;
			sum += buf[size_t(i)];
			uint8_t* m = mask + (size_t(y) * pw + i) * 4;
			m[0] = 0xFF;
			m[1] = v;
			m[2] = v;
			m[3] = v;
		}
		if (y >= radius)
			for (int i = 0; i < pw; i++)
				buf[size_t(radius + i)] -= alphaOn(y - radius, i);
	}
	return 0;
}

/* Table access for pinning the generated tables against the reference's. */
const void* nebc7_oracle_table(int denoise, int id, int* size)
{
	const LevelTables& t = GetLevelTables(denoise);
	const void* p = nullptr;
	int s = 0;
	switch (id)
	{
	case 0: p = t.d2v8; s = 256 * 65536; break;
	case 1: p = t.d2v7; s = 256 * 16384; break;
	case 2: p = t.d2v6; s = 256 * 4096; break;
	case 3: p = t.d2v5; s = 256 * 1024; break;
	case 4: p = t.c2v8; s = 256 * 256 * 2; break;
	case 5: p = t.c2v6; s = 256 * 64 * 2; break;
	case 6: p = t.c2v5; s = 256 * 32 * 2; break;
	case 7: p = t.d3v7s; s = 256 * 16384; break;
	case 8: p = t.d3v6; s = 256 * 4096; break;
	case 9: p = t.d3v5; s = 256 * 1024; break;
	case 10: p = t.c3v7s; s = 256 * 128 * 2; break;
	case 11: p = t.c3v5; s = 256 * 32 * 2; break;
	case 12: p = t.d4h; s = 256 * 32768; break;
	case 13: p = t.d2h; s = 256 * 32768; break;
	}
	if (size)
		*size = s;
	return p;
}

} // extern "C"
