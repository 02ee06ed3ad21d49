/*
 * Test infrastructure: the reference encoder with its draft chain reduced to
 * the Mode6Index2 pass, for the "Mode6Index2 fast" run.  The reference has
 * no switch for it: Mode6Index2::CompressBlockFast is the first pass of its
 * draft chain (src/Bc7Core.cpp:1546-1552), followed by the Mode6, 4, 5, 7
 * fast passes (:1554-1574) and, for opaque blocks, the Mode3, 1, 2, 0 fast
 * passes (:1577-1597).
 *
 * oracle/build_ref.sh compiles the reference's Bc7CoreMode{0..7}.cpp for
 * this variant with -DCompressBlockFast=CompressBlockFastOff, so their own
 * fast passes get another name, and links these empty passes under the
 * reference's names instead.  Bc7Core.cpp and Bc7CoreMode6Index2.cpp are
 * compiled unchanged.  Run with doDraft set and doNormal / doSlow clear (the
 * CLI's /draft), the reference then runs exactly: Mode6Index2's fast pass,
 * the final pack, and the self-check.  Sources are read unmodified.
 */
#include "Bc7Core.h"

namespace Mode0 { void CompressBlockFast(Cell&) noexcept {} }
namespace Mode1 { void CompressBlockFast(Cell&) noexcept {} }
namespace Mode2 { void CompressBlockFast(Cell&) noexcept {} }
namespace Mode3 { void CompressBlockFast(Cell&) noexcept {} }
namespace Mode4 { void CompressBlockFast(Cell&) noexcept {} }
namespace Mode5 { void CompressBlockFast(Cell&) noexcept {} }
namespace Mode6 { void CompressBlockFast(Cell&) noexcept {} }
namespace Mode7 { void CompressBlockFast(Cell&) noexcept {} }
