/*
 * In-memory IO for the reference's command-line build (test infrastructure
 * only; see ref_cli_shim.h) and a C entry that runs its CLI driver
 * Bc7MainWithArgs (src/Bc7Compress.cpp:267) with the debug outputs on:
 *
 *   /map  -- the partition visualisation (src/Bc7Compress.cpp:131-265,
 *            :532-537): the blocks rewritten by VisualizePartitionsGRB and
 *            decoded;
 *   /bad  -- the glitch map (src/Worker.cpp:309-451, src/Bc7Compress.cpp:
 *            525-529): each block whose decoded pixels differ from the
 *            source by more than the per-channel steps keeps its source
 *            pixels, the others are zero.
 *
 * Images are BGRA, top-down rows, padded to a multiple of 4.
 */
#include <string.h>

#include <string>
#include <vector>

int Bc7MainWithArgs(const struct IBc7Core& bc7Core, const std::vector<std::string>& args);
bool GetBc7Core(void* bc7Core);

std::atomic<int> gNebc7RefCliSelfCheckFailures{0};

namespace {

struct CliImage
{
	const uint8_t* bgra = nullptr;
	int w = 0, h = 0;
	uint8_t* blocks = nullptr;
	int blocksSize = 0;
	uint8_t* map = nullptr;       /* padded w * h * 4, or null */
	uint8_t* bad = nullptr;       /* padded w * h * 4, or null */
	int written = 0;              /* bit 0: blocks, 1: map, 2: bad */
};

CliImage gCli;

} // namespace

bool ReadImage(const char*, uint8_t*& pixels, int& width, int& height, bool)
{
	if (!gCli.bgra)
		return false;
	width = gCli.w;
	height = gCli.h;
	pixels = new uint8_t[size_t(width) * size_t(height) * 4];
	memcpy(pixels, gCli.bgra, size_t(width) * size_t(height) * 4);
	return true;
}

void WriteImage(const char* dst_name, const uint8_t* pixels, int w, int h, bool)
{
	const std::string name = dst_name ? dst_name : "";
	uint8_t* to = name == "map.png" ? gCli.map : (name == "bad.png" ? gCli.bad : nullptr);
	if (to)
	{
		memcpy(to, pixels, size_t(w) * size_t(h) * 4);
		gCli.written |= name == "map.png" ? 2 : 4;
	}
}

void LoadBc7(const char*, int, uint8_t*, int)
{
}

void SaveBc7(const char*, const uint8_t*, int, const uint8_t* buffer, int size)
{
	if (gCli.blocks && size <= gCli.blocksSize)
	{
		memcpy(gCli.blocks, buffer, size_t(size));
		gCli.written |= 1;
	}
}

#include "Bc7Core.h"

extern "C" int nebc7_ref_cli(const uint8_t* bgra, int w, int h, const char* flags, uint8_t* blocks, int blocksSize,
	uint8_t* map, uint8_t* bad)
{
	gCli = CliImage();
	gCli.bgra = bgra;
	gCli.w = w;
	gCli.h = h;
	gCli.blocks = blocks;
	gCli.blocksSize = blocksSize;
	gCli.map = map;
	gCli.bad = bad;

	std::vector<std::string> args;
	const std::string f = flags ? flags : "";
	for (size_t p = 0; p < f.size();)
	{
		size_t q = f.find(' ', p);
		if (q == std::string::npos)
			q = f.size();
		if (q > p)
			args.emplace_back(f.substr(p, q - p));
		p = q + 1;
	}
	if (map)
	{
		args.emplace_back("/map");
		args.emplace_back("map.png");
	}
	if (bad)
	{
		args.emplace_back("/bad");
		args.emplace_back("bad.png");
	}
	args.emplace_back("memory.png");
	args.emplace_back("memory.ktx");

	IBc7Core core{};
	if (!GetBc7Core(&core))
		return -2;
	const int failures = gNebc7RefCliSelfCheckFailures.load();
	const int rc = Bc7MainWithArgs(core, args);
	if (gNebc7RefCliSelfCheckFailures.load() != failures)
		return -3;
	return rc != 0 ? rc : gCli.written;
}
