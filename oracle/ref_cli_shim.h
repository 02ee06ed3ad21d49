/*
 * Force-included header for the reference's command-line build (test
 * infrastructure only): all reference sources compiled with their own
 * configuration (src/Bc7Mode.h as shipped: AVX2, FMA, self-check, kDenoise
 * 1, kDenoiseStep 9) and without OPTION_LIBRARY, so that the CLI driver's
 * /map and /bad steps (src/Bc7Compress.cpp:520-537) and the real job pool
 * (src/Worker.cpp) are compiled.  Sources are read unmodified.
 *
 * Outside Win32 the reference needs two things it does not ship: boost's
 * thread with a stack-size attribute (src/Worker.cpp:224-226) and the image
 * IO declarations of src/IO.h, which that header provides for Win32 only.
 * Both are supplied here (with <mutex>, which boost's headers would bring for
 * the Worker's std::mutex); the IO itself is in-memory (ref_cli_harness.cpp).
 */
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <atomic>
#include <functional>
#include <mutex>
#include <thread>

namespace boost {

/* std::thread under boost::thread's spelling; the stack-size request
   (1 MB) is below the default thread stack on Linux (8 MB). */
class thread
{
public:
	class attributes
	{
	public:
		void set_stack_size(size_t) {}
	};

	template<class F>
	thread(const attributes&, F f) : t_(f) {}

	void detach() { t_.detach(); }

private:
	std::thread t_;
};

using std::bind;

} // namespace boost

/* MSVC's breakpoint intrinsic in the self-check (src/Bc7Core.cpp:1799-1807):
   a mismatch is counted, not trapped. */
extern std::atomic<int> gNebc7RefCliSelfCheckFailures;
#define __debugbreak() (gNebc7RefCliSelfCheckFailures++)

bool ReadImage(const char* src_name, uint8_t*& pixels, int& width, int& height, bool flip);
void WriteImage(const char* dst_name, const uint8_t* pixels, int w, int h, bool flip);
void LoadBc7(const char* name, int position, uint8_t* buffer, int size);
void SaveBc7(const char* name, const uint8_t* head, int position, const uint8_t* buffer, int size);
