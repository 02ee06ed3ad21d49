/*
 * Force-included configuration header for building the reference encoder
 * sources unmodified on Linux/g++ (test infrastructure only: the reference
 * build is the oracle that pins the port in this directory and generates the
 * golden fixtures under tests/golden; nothing in the product links it).
 *
 * The reference's pch.h includes nothing when OPTION_LIBRARY is defined and
 * nothing includes Bc7Mode.h, so this header supplies what those two files
 * would (src/pch.h:1-47, src/Bc7Mode.h:1-35): the ISA options, the
 * kDenoise / kDenoiseStep preset, kWeightLimit, the channel-weight externs,
 * the intrinsics headers and the inlining macros.  The preset is chosen with
 * -DNEBC7_REF_DENOISE=<0|1> -DNEBC7_REF_DENOISE_STEP=<0|9>.
 *
 * The CLI driver (src/Bc7Compress.cpp) is compiled too so that the
 * reference's own padding, mask and flag handling produce the fixtures; its
 * Win32 image IO is replaced by the in-memory IO in ref_harness.cpp, whose
 * declarations follow.
 */
#pragma once

#include <stdint.h>
#include <string.h>
#include <math.h>
#include <stdio.h>
#include <immintrin.h>
#include <atomic>
#include <mutex>

#define OPTION_AVX2
#define OPTION_FMA
#define OPTION_SELFCHECK

#ifndef NEBC7_REF_DENOISE
#define NEBC7_REF_DENOISE 1
#endif
#ifndef NEBC7_REF_DENOISE_STEP
#define NEBC7_REF_DENOISE_STEP 9
#endif

enum { kDenoise = NEBC7_REF_DENOISE, kDenoiseStep = NEBC7_REF_DENOISE_STEP };
enum { kDenoiseShift = kDenoise ? kDenoise : 1 };

constexpr int kWeightLimit = 1000;
extern int gWeightAlpha, gWeightGreen, gWeightRed, gWeightBlue;
extern int gWeightColor, gWeightColorAlpha;

#define ALWAYS_INLINED __attribute__((always_inline)) inline
#define NOTINLINED __attribute__((noinline))
#define INLINED ALWAYS_INLINED

extern int gNebc7RefQuiet;
#define PRINTF(...) do { if (!gNebc7RefQuiet) { printf(__VA_ARGS__); printf("\n"); } } while (0)

/* A self-check mismatch (src/Bc7Core.cpp:1799-1807) is counted, not trapped. */
extern std::atomic<int> gNebc7RefSelfCheckFailures;
#define __debugbreak() (gNebc7RefSelfCheckFailures++)

/* In-memory replacements for the Win32 IO of src/IO.h:7-11. */
bool ReadImage(const char* src_name, uint8_t*& pixels, int& width, int& height, bool flip);
void LoadBc7(const char* name, int position, uint8_t* buffer, int size);
void SaveBc7(const char* name, const uint8_t* head, int position, const uint8_t* buffer, int size);
