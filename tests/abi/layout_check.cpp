/*
 * Compile-time check (test support, CPU only): the structures of
 * include/nebc7_gb300.h have the machine layout of the reference's own
 * (src/Bc7Core.h:25-35 BlockSSIM, :294-322 WorkerItem and IBc7Core).
 *
 * Built with g++ -fsyntax-only against the reference's headers, with the
 * oracle's force-included configuration header (oracle/ref_shim.h) standing
 * in for the reference's pch.h.  The library's header is read inside a
 * namespace of its own, because it declares the same type names.
 */
#include <cstddef>
#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include <type_traits>

#include "Bc7Core.h"

namespace lib {
#include "nebc7_gb300.h"
}

#define SAME_FIELD(T, f) \
	static_assert(offsetof(lib::T, f) == offsetof(::T, f), #T "::" #f " offset"); \
	static_assert(sizeof(lib::T::f) == sizeof(::T::f), #T "::" #f " size")

static_assert(sizeof(lib::WorkerItem) == sizeof(::WorkerItem), "WorkerItem size");
static_assert(alignof(lib::WorkerItem) == alignof(::WorkerItem), "WorkerItem alignment");
SAME_FIELD(WorkerItem, _Output);
SAME_FIELD(WorkerItem, _Cell);
SAME_FIELD(WorkerItem, _Mask);

static_assert(sizeof(lib::BlockSSIM) == sizeof(::BlockSSIM), "BlockSSIM size");
static_assert(alignof(lib::BlockSSIM) == alignof(::BlockSSIM), "BlockSSIM alignment");
SAME_FIELD(BlockSSIM, Alpha);
SAME_FIELD(BlockSSIM, Color);

static_assert(sizeof(lib::IBc7Core) == sizeof(::IBc7Core), "IBc7Core size");
SAME_FIELD(IBc7Core, pInitTables);
SAME_FIELD(IBc7Core, pDecompress);
SAME_FIELD(IBc7Core, pCompress);
SAME_FIELD(IBc7Core, pGetWeightAlpha);
SAME_FIELD(IBc7Core, pGetWeightColor);

/* The entry signatures: the same parameter list, where the reference's
   C++ references (int64_t&, BlockSSIM&) are pointers here -- the same
   machine-level argument on every C++ ABI this builds for. */
static_assert(std::is_same<::PInitTables, lib::PInitTables>::value, "PInitTables");
static_assert(std::is_same<decltype(std::declval<::PGetWeight>()()), decltype(std::declval<lib::PGetWeight>()())>::value,
	"PGetWeight result");
static_assert(std::is_same<::PBlockKernel,
	void (*)(const ::WorkerItem*, const ::WorkerItem*, int, int64_t&, int64_t&, ::BlockSSIM&) noexcept>::value,
	"the reference's PBlockKernel");
static_assert(std::is_same<lib::PBlockKernel,
	void (*)(const lib::WorkerItem*, const lib::WorkerItem*, int, int64_t*, int64_t*, lib::BlockSSIM*)>::value,
	"the library's PBlockKernel");
static_assert(sizeof(int64_t&) == sizeof(int64_t) && sizeof(int64_t*) == sizeof(void*), "reference-as-pointer");
