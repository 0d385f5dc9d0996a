// Index guards of the bounds-checked debug build.
//
// Built with -DWENOFD_BOUNDS_CHECK (build.py --bounds-check), every guarded
// index -- of the state, flag, table and work arrays in global memory, of the
// tiles in shared memory, and the TMA boxes' first coordinates -- is tested
// against its extent before the access.  An index out of range is not used:
// the access goes to element 0 of the same array instead (a guarded stencil
// span to its first element), and the device's guard record counts the
// violation and keeps the first one: the source site (file-name hash and
// line), the index and the extent.  The host reads the record with
// wenofd_bounds_report.  In the release build the guards are the bare index
// and the record pointer stays null.
//
// This takes the place of the reference's assert-checked Array1D/Array2D
// indexing (utils/array.h:273-303, 552-583) for the device code.
#pragma once

#include "wenofd_internal.h"

namespace wenofd {

// FNV-1a hash of a path's base name (the host maps it back to the name).
__host__ __device__ constexpr unsigned guard_file_hash(const char *path) {
  const char *b = path;
  for (const char *p = path; *p; ++p)
    if (*p == '/' || *p == '\\') b = p + 1;
  unsigned h = 2166136261u;
  for (const char *p = b; *p; ++p) h = (h ^ static_cast<unsigned char>(*p)) * 16777619u;
  return h;
}
__host__ __device__ constexpr unsigned long long guard_site(const char *path, int line) {
  return (static_cast<unsigned long long>(guard_file_hash(path)) << 32) | static_cast<unsigned>(line);
}

// Layout of the device guard record (unsigned long long words).
enum { kGuardCount = 0, kGuardSite = 1, kGuardIndex = 2, kGuardExtent = 3, kGuardWords = 4 };

#ifdef __CUDACC__
namespace dev {

// The slow path, out of line so the guards stay small.
template <int = 0>
__device__ __noinline__ void guard_hit(unsigned long long *rec, unsigned long long site, long long i, long long n) {
  if (rec == nullptr) return;
  if (atomicAdd(rec + kGuardCount, 1ull) == 0ull) {
    rec[kGuardSite] = site;
    rec[kGuardIndex] = static_cast<unsigned long long>(i);
    rec[kGuardExtent] = static_cast<unsigned long long>(n);
  }
}

// i if `ok` and 0 <= i < n, else 0 (recorded).
template <unsigned long long SITE, typename I>
__device__ __forceinline__ I guard_ix(unsigned long long *rec, bool ok, I i, long long n) {
  if (ok && static_cast<unsigned long long>(static_cast<long long>(i)) < static_cast<unsigned long long>(n)) return i;
  guard_hit(rec, SITE, static_cast<long long>(i), n);
  return I(0);
}

// first if the whole span first..last lies in [0, n), else 0 (recorded with
// the end that fell outside).
template <unsigned long long SITE, typename I>
__device__ __forceinline__ I guard_span(unsigned long long *rec, I first, I last, long long n) {
  const bool lo = static_cast<unsigned long long>(static_cast<long long>(first)) < static_cast<unsigned long long>(n);
  const bool hi = static_cast<unsigned long long>(static_cast<long long>(last)) < static_cast<unsigned long long>(n);
  if (lo && hi) return first;
  guard_hit(rec, SITE, static_cast<long long>(lo ? last : first), n);
  return I(0);
}

// Like guard_ix for an access that happens only when `active`: an inactive
// index is not checked (its value is unused) and comes back as 0.
template <unsigned long long SITE, typename I>
__device__ __forceinline__ I guard_ix_if(unsigned long long *rec, bool active, bool ok, I i, long long n) {
  if (!active) return I(0);
  return guard_ix<SITE>(rec, ok, i, n);
}

// cond, recording (i, n) when it fails.
template <unsigned long long SITE>
__device__ __forceinline__ bool guard_require(unsigned long long *rec, bool cond, long long i, long long n) {
  if (!cond) guard_hit(rec, SITE, i, n);
  return cond;
}

}  // namespace dev
#endif  // __CUDACC__

}  // namespace wenofd

#if defined(WENOFD_BOUNDS_CHECK) && defined(__CUDACC__)
#define WENOFD_IX(rec, i, n) \
  (::wenofd::dev::guard_ix<::wenofd::guard_site(__FILE__, __LINE__)>((rec), true, (i), (long long)(n)))
// i, guarded with an extra condition (e.g. per-dimension ranges)
#define WENOFD_IXC(rec, ok, i, n) \
  (::wenofd::dev::guard_ix<::wenofd::guard_site(__FILE__, __LINE__)>((rec), (ok), (i), (long long)(n)))
// i for an access made only when `active` (not checked otherwise)
#define WENOFD_IXIF(rec, active, ok, i, n) \
  (::wenofd::dev::guard_ix_if<::wenofd::guard_site(__FILE__, __LINE__)>((rec), (active), (ok), (i), (long long)(n)))
#define WENOFD_SPAN(rec, first, last, n) \
  (::wenofd::dev::guard_span<::wenofd::guard_site(__FILE__, __LINE__)>((rec), (first), (last), (long long)(n)))
#define WENOFD_REQUIRE(rec, cond, i, n) \
  (::wenofd::dev::guard_require<::wenofd::guard_site(__FILE__, __LINE__)>((rec), (cond), (long long)(i), (long long)(n)))
#else
#define WENOFD_IX(rec, i, n) (i)
#define WENOFD_IXC(rec, ok, i, n) (i)
#define WENOFD_IXIF(rec, active, ok, i, n) (i)
#define WENOFD_SPAN(rec, first, last, n) (first)
#define WENOFD_REQUIRE(rec, cond, i, n) true
#endif

// Offsets within one state plane: interior node (i, j), 0-based, and
// ghosted node (ei, ej) (columns up to the pitch: the row padding is
// allocated).  Each is guarded per dimension and against the plane.
#define WENOFD_NODE(g, i, j)                                                                          \
  WENOFD_IXC((g).guard, unsigned(i) < unsigned((g).nx) && unsigned(j) < unsigned((g).ny),            \
             (long long)(::wenofd::kGhost + (i)) * (g).pitch + (::wenofd::kGhost + (j)), (g).plane)
#define WENOFD_GNODE(g, ei, ej)                                                                       \
  WENOFD_IXC((g).guard, unsigned(ei) < unsigned((g).nxt) && unsigned(ej) < unsigned((g).pitch),      \
             (long long)(ei) * (g).pitch + (ej), (g).plane)
// WENOFD_GNODE for an access made only when `active`.
#define WENOFD_GNODE_IF(g, active, ei, ej)                                                            \
  WENOFD_IXIF((g).guard, (active), unsigned(ei) < unsigned((g).nxt) && unsigned(ej) < unsigned((g).pitch), \
              (long long)(ei) * (g).pitch + (ej), (g).plane)
// An index into a whole state array [4][nxt][pitch].
#define WENOFD_STATE(g, k) WENOFD_IX((g).guard, (k), 4 * (g).plane)
// Entries of the SPECIAL boundary table (8 nxt + 8 nyt doubles).
#define WENOFD_SPECIAL(g, k) WENOFD_IX((g).guard, (k), 8LL * (g).nxt + 8LL * (g).nyt)
