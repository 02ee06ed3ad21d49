/*
 * CPU oracle for the BC7 block encoder -- table generation (test
 * infrastructure only; see port_tables.h).  Restates reference
 * src/Bc7Tables.cpp; each block cites the lines it follows.
 */
#include "port_tables.h"

#include <mutex>
#include <stdlib.h>
#include <string.h>

namespace nebc7_oracle {

/* BPTC interpolation weights (src/Bc7Tables.cpp:7-48). */
const int kInterp2[4] = { 0, 21, 43, 64 };
const int kInterp3[8] = { 0, 9, 18, 27, 37, 46, 55, 64 };
const int kInterp4[16] = { 0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64 };

/* BPTC two-subset partitions (src/Bc7Tables.cpp:171), 2 bits per pixel. */
const uint32_t kPartition2[64] = {
	0x50505050u, 0x40404040u, 0x54545454u, 0x54505040u, 0x50404000u, 0x55545450u, 0x55545040u, 0x54504000u,
	0x50400000u, 0x55555450u, 0x55544000u, 0x54400000u, 0x55555440u, 0x55550000u, 0x55555500u, 0x55000000u,
	0x55150100u, 0x00004054u, 0x15010000u, 0x00405054u, 0x00004050u, 0x15050100u, 0x05010000u, 0x40505054u,
	0x00404050u, 0x05010100u, 0x14141414u, 0x05141450u, 0x01155440u, 0x00555500u, 0x15014054u, 0x05414150u,
	0x44444444u, 0x55005500u, 0x11441144u, 0x05055050u, 0x05500550u, 0x11114444u, 0x41144114u, 0x44111144u,
	0x15055054u, 0x01055040u, 0x05041050u, 0x05455150u, 0x14414114u, 0x50050550u, 0x41411414u, 0x00141400u,
	0x00041504u, 0x00105410u, 0x10541000u, 0x04150400u, 0x50410514u, 0x41051450u, 0x05415014u, 0x14054150u,
	0x41050514u, 0x41505014u, 0x40011554u, 0x54150140u, 0x50505500u, 0x00555050u, 0x15151010u, 0x54540404u,
};

/* BPTC three-subset partitions (src/Bc7Tables.cpp:242), 2 bits per pixel. */
const uint32_t kPartition3[64] = {
	0xAA685050u, 0x6A5A5040u, 0x5A5A4200u, 0x5450A0A8u, 0xA5A50000u, 0xA0A05050u, 0x5555A0A0u, 0x5A5A5050u,
	0xAA550000u, 0xAA555500u, 0xAAAA5500u, 0x90909090u, 0x94949494u, 0xA4A4A4A4u, 0xA9A59450u, 0x2A0A4250u,
	0xA5945040u, 0x0A425054u, 0xA5A5A500u, 0x55A0A0A0u, 0xA8A85454u, 0x6A6A4040u, 0xA4A45000u, 0x1A1A0500u,
	0x0050A4A4u, 0xAAA59090u, 0x14696914u, 0x69691400u, 0xA08585A0u, 0xAA821414u, 0x50A4A450u, 0x6A5A0200u,
	0xA9A58000u, 0x5090A0A8u, 0xA8A09050u, 0x24242424u, 0x00AA5500u, 0x24924924u, 0x24499224u, 0x50A50A50u,
	0x500AA550u, 0xAAAA4444u, 0x66660000u, 0xA5A0A5A0u, 0x50A050A0u, 0x69286928u, 0x44AAAA44u, 0x66666600u,
	0xAA444444u, 0x54A854A8u, 0x95809580u, 0x96969600u, 0xA85454A8u, 0x80959580u, 0xAA141414u, 0x96960000u,
	0xAAAA1414u, 0xA05050A0u, 0xA0A5A5A0u, 0x96000000u, 0x40804080u, 0xA9A8A9A8u, 0xAAAAAA44u, 0x2A4A5254u,
};

/* BPTC anchor indices (src/Bc7Tables.cpp:313, 325, 337). */
const uint8_t kAnchor2of2[64] = {
	15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 2, 8, 2, 2, 8, 8, 15, 2, 8, 2, 2, 8, 8, 2, 2,
	15, 15, 6, 8, 2, 8, 15, 15, 2, 8, 2, 2, 2, 15, 15, 6, 6, 2, 6, 8, 15, 15, 2, 2, 15, 15, 15, 15, 15, 2, 2, 15,
};
const uint8_t kAnchor2of3[64] = {
	3, 3, 15, 15, 8, 3, 15, 15, 8, 8, 6, 6, 6, 5, 3, 3, 3, 3, 8, 15, 3, 3, 6, 10, 5, 8, 8, 6, 8, 5, 15, 15,
	8, 15, 3, 5, 6, 10, 8, 15, 15, 3, 15, 5, 15, 15, 15, 15, 3, 15, 5, 5, 5, 8, 5, 10, 5, 10, 8, 13, 15, 12, 3, 3,
};
const uint8_t kAnchor3of3[64] = {
	15, 8, 8, 3, 15, 15, 3, 8, 15, 15, 15, 15, 15, 15, 15, 8, 15, 8, 15, 3, 15, 8, 15, 8, 3, 15, 6, 10, 15, 15, 10, 8,
	15, 3, 15, 10, 10, 8, 9, 10, 6, 15, 8, 15, 3, 6, 6, 8, 15, 3, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 3, 15, 15, 8,
};

const int kRotationsMode4[8] = { 0 + 4, 0, 2 + 4, 2, 1 + 4, 1, 3 + 4, 3 };
const int kRotationsMode5[4] = { 0, 2, 1, 3 };

static Selection BuildSelection()
{
	Selection s;
	for (int p = 0; p < 64; p++)
	{
		/* src/Bc7Tables.cpp:352-367 */
		uint8_t a = kAnchor2of3[p], b = kAnchor3of3[p];
		if (a > b)
		{
			uint8_t c = a; a = b; b = c;
		}
		s.anchorLow3[p] = a;
		s.anchorHigh3[p] = b;

		/* src/Bc7Tables.cpp:381-419: anchor first, then the other pixels in order;
		   low nibble = count, then one nibble per pixel index. */
		{
			const uint64_t stop2 = kAnchor2of2[p];
			uint64_t i1 = 0, i2 = stop2;
			int n1 = 1, n2 = 1;
			for (uint64_t i = 1; i < 16; i++)
			{
				if (((kPartition2[p] >> (2 * i)) & 3) == 0)
				{
					i1 |= i << (n1 << 2);
					n1++;
				}
				else if (i != stop2)
				{
					i2 |= i << (n2 << 2);
					n2++;
				}
			}
			s.sel12[p] = (i1 << 4) | uint64_t(n1);
			s.sel22[p] = (i2 << 4) | uint64_t(n2);
		}
		/* src/Bc7Tables.cpp:421-473 */
		{
			const uint64_t stop2 = kAnchor2of3[p], stop3 = kAnchor3of3[p];
			uint64_t i1 = 0, i2 = stop2, i3 = stop3;
			int n1 = 1, n2 = 1, n3 = 1;
			for (uint64_t i = 1; i < 16; i++)
			{
				uint32_t sub = (kPartition3[p] >> (2 * i)) & 3;
				if (sub == 0)
				{
					i1 |= i << (n1 << 2);
					n1++;
				}
				else if (sub == 1)
				{
					if (i != stop2)
					{
						i2 |= i << (n2 << 2);
						n2++;
					}
				}
				else if (i != stop3)
				{
					i3 |= i << (n3 << 2);
					n3++;
				}
			}
			s.sel13[p] = (i1 << 4) | uint64_t(n1);
			s.sel23[p] = (i2 << 4) | uint64_t(n2);
			s.sel33[p] = (i3 << 4) | uint64_t(n3);
		}
	}
	return s;
}

const Selection& GetSelection()
{
	static const Selection s = BuildSelection();
	return s;
}

/* The per-pixel error quantiser q(|d|): kDenoise=1 drops the least bit, kDenoise=0
   saturates at 127 (the adds_epu8 doubling then >>1 of src/Bc7Tables.cpp:623-628). */
static inline int Quant(int d, int denoise)
{
	d = d < 0 ? -d : d;
	if (denoise)
		return d >> denoise;
	return d > 127 ? 127 : d;
}

/* min over levels of |((64-w) cL + w cH + 32) >> 6 - x|, quantised,
   for all x and c = (cH << 8) + cL (src/Bc7Tables.cpp:604-633). */
static void BuildFull(uint8_t* out, const int* w, int levels, int denoise, int clamp15, int nibbles)
{
	for (int c = 0; c < 0x10000; c++)
	{
		const int cL = c & 0xFF, cH = c >> 8;
		int v[16];
		for (int k = 0; k < levels; k++)
			v[k] = (cL * (64 - w[k]) + cH * w[k] + 32) >> 6;
		for (int x = 0; x < 0x100; x++)
		{
			int best = 0x7FFF;
			for (int k = 0; k < levels; k++)
			{
				int d = v[k] - x;
				d = d < 0 ? -d : d;
				best = d < best ? d : best;
			}
			int q = Quant(best, denoise);
			if (clamp15 && q > 15)
				q = 15;
			if (nibbles)
				out[size_t(x) * 0x8000 + (c >> 1)] |= uint8_t(q << ((c & 1) << 2));
			else
				out[size_t(x) * 0x10000 + c] = uint8_t(q);
		}
	}
}

/* src/Bc7Tables.cpp:497-516: keep the pairs whose both endpoints are
   bits-bit values expanded by bit replication. */
static void Reduce(const uint8_t* full, uint8_t* p, int bits)
{
	const int step = 1 << (8 - bits);
	for (int x = 0; x < 0x100; x++)
		for (int iH = 0; iH < 0x100; iH += step)
		{
			const int cH = (iH + (iH >> bits)) << 8;
			for (int iL = 0; iL < 0x100; iL += step)
				*p++ = full[size_t(x) * 0x10000 + cH + iL + (iL >> bits)];
		}
}

/* src/Bc7Tables.cpp:518-535: shared p-bit pairs with different parity are invalid. */
static void FilterShared(uint8_t* p, int bits)
{
	const int n = 1 << bits;
	for (int x = 0; x < 0x100; x++)
		for (int iH = 0; iH < n; iH++)
		{
			for (int iL = (iH & 1) ^ 1; iL < n; iL += 2)
				p[iL] = 0xFF;
			p += n;
		}
}

/* src/Bc7Tables.cpp:537-581: squared minimum over the row prefix [0, iH|31]. */
static void Cut(const uint8_t* table, uint16_t* tower, int bits)
{
	const int n = 1 << bits;
	for (int x = 0; x < 0x100; x++)
		for (int iH = 0; iH < n; iH++)
		{
			const uint8_t* row = table + size_t(x) * n * n + size_t(iH) * n;
			int cut = 0xFFFF;
			for (int iL = 0, hL = iH | 31; iL <= hL; iL++)
				cut = row[iL] < cut ? row[iL] : cut;
			tower[size_t(x) * n + iH] = uint16_t(cut * cut);
		}
}

static LevelTables BuildLevels(int denoise)
{
	LevelTables t;
	t.denoise = denoise;
	auto u8 = [](size_t n) { return static_cast<uint8_t*>(calloc(n, 1)); };
	auto u16 = [](size_t n) { return static_cast<uint16_t*>(calloc(n, 2)); };

	t.d2v8 = u8(size_t(256) * 65536);
	t.d2v7 = u8(size_t(256) * 16384);
	t.d2v6 = u8(size_t(256) * 4096);
	t.d2v5 = u8(size_t(256) * 1024);
	t.c2v8 = u16(size_t(256) * 256);
	t.c2v6 = u16(size_t(256) * 64);
	t.c2v5 = u16(size_t(256) * 32);
	t.d3v7s = u8(size_t(256) * 16384);
	t.d3v6 = u8(size_t(256) * 4096);
	t.d3v5 = u8(size_t(256) * 1024);
	t.c3v7s = u16(size_t(256) * 128);
	t.c3v5 = u16(size_t(256) * 32);
	t.d4h = u8(size_t(256) * 32768);
	t.d2h = u8(size_t(256) * 32768);

	/* 3-bit index (src/Bc7Tables.cpp:587-641) */
	{
		uint8_t* d3v8 = u8(size_t(256) * 65536);
		BuildFull(d3v8, kInterp3, 8, denoise, 0, 0);
		Reduce(d3v8, t.d3v7s, 7);
		FilterShared(t.d3v7s, 7);
		Reduce(d3v8, t.d3v6, 6);
		Reduce(d3v8, t.d3v5, 5);
		Cut(t.d3v7s, t.c3v7s, 7);
		Cut(t.d3v5, t.c3v5, 5);
		free(d3v8);
	}
	/* 2-bit index (src/Bc7Tables.cpp:643-692) */
	BuildFull(t.d2v8, kInterp2, 4, denoise, 0, 0);
	Reduce(t.d2v8, t.d2v7, 7);
	Reduce(t.d2v8, t.d2v6, 6);
	Reduce(t.d2v8, t.d2v5, 5);
	Cut(t.d2v8, t.c2v8, 8);
	Cut(t.d2v6, t.c2v6, 6);
	Cut(t.d2v5, t.c2v5, 5);
	/* 4-bit index, nibbles clamped to 15 (src/Bc7Tables.cpp:694-761) */
	BuildFull(t.d4h, kInterp4, 16, denoise, 1, 1);
	/* 2-bit subset of the 4-bit index (src/Bc7Tables.cpp:763-776) */
	for (int x = 0; x < 0x100; x++)
		for (int c = 0; c < 0x10000; c++)
		{
			int v = t.d2v8[size_t(x) * 0x10000 + c];
			v = v > 15 ? 15 : v;
			t.d2h[size_t(x) * 0x8000 + (c >> 1)] |= uint8_t(v << ((c & 1) << 2));
		}
	return t;
}

const LevelTables& GetLevelTables(int denoise)
{
	static std::once_flag once[2];
	static LevelTables tables[2];
	const int i = denoise ? 1 : 0;
	std::call_once(once[i], [i]() { tables[i] = BuildLevels(i); });
	return tables[i];
}

} // namespace nebc7_oracle
