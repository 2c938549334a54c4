// gw_layout.h -- device-resident layout of the packed event/dial cache.
//
// The reference keeps one table per dial type and multiplies each dial into
// the event weight with a 64-bit CAS loop (CacheAtomicMult.h:12-47), then sums
// bins with log2(max occupancy) full passes (CacheRecursiveSums.cpp:282-352).
// Here the events are sorted by histogram bin and cut into TILES.  A tile is a
// contiguous run of bin-sorted events together with all of their dials; its
// dial payload is one contiguous, 16-byte aligned byte range, so one bulk copy
// (TMA) moves it into shared memory.  Inside a tile the dials are ordered by
// type (so a warp evaluates one code path at a time) and each dial carries its
// SLOT: its position in event-major order, which is where its value is
// written for the segmented per-event product.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define GW_HD __host__ __device__ __forceinline__
#else
#define GW_HD inline
#endif

namespace gw {

constexpr int kMaxTileDials = 1023;   // slot field is 10 bits
constexpr int kMaxTileEvents = 256;   // one event per thread in the plain kernel
constexpr int kMaxLocalBins = 4;      // bins spanned by one tile (bin - bin0 < 4)
constexpr int kMaxPayloadElems = 8191; // 13-bit element offset
constexpr int kMaxKnots = 31;         // 5-bit count field
constexpr int kTypeCount = 11;
constexpr int kMaxGrids = 16384;      // knot grids of the grid form (p0 field of the header)

// Dial type codes (same numbering as the public GW_DIAL_* enum).
enum : int {
  kNone = 0,
  kNorm = 1,
  kMonotonic = 2,
  kUniform = 3,
  kGeneral = 4,
  kCompact = 5,
  kGraph = 6,
  kBilinear = 7,
  kBicubic = 8,
  kTabulated = 9,
  kKriged = 10,
  // Header-only code (never a public dial type): a monotonic, compact or
  // uniform spline of the grid form, whose knot grid (parameter, first knot,
  // step, knot count) it shares with other dials.  Its header's p0 field holds
  // the grid's index, its payload the per-interval cubic coefficients alone.
  kGrid = 11
};

// 64-bit dial header:
//   [0,4)   type
//   [4,9)   n      knots / points / kriging weights (0 for norm, surfaces)
//   [9,19)  slot   event-major position inside the tile
//   [19,32) off    payload offset inside the tile, in elements of the payload type
//   [32,48) p0     parameter index (table index for table dials)
//   [48,64) p1     second parameter of surface dials
GW_HD uint64_t make_header(int type, int n, int slot, int off, int p0, int p1) {
  return (uint64_t)(type & 0xF) | ((uint64_t)(n & 0x1F) << 4) |
         ((uint64_t)(slot & 0x3FF) << 9) | ((uint64_t)(off & 0x1FFF) << 19) |
         ((uint64_t)(p0 & 0xFFFF) << 32) | ((uint64_t)(p1 & 0xFFFF) << 48);
}
GW_HD int hdr_type(uint64_t h) { return (int)(h & 0xF); }
GW_HD int hdr_n(uint64_t h) { return (int)((h >> 4) & 0x1F); }
GW_HD int hdr_slot(uint64_t h) { return (int)((h >> 9) & 0x3FF); }
GW_HD int hdr_off(uint64_t h) { return (int)((h >> 19) & 0x1FFF); }
GW_HD int hdr_p0(uint64_t h) { return (int)((h >> 32) & 0xFFFF); }
GW_HD int hdr_p1(uint64_t h) { return (int)((h >> 48) & 0xFFFF); }

// Relative work of one dial in the lanes-over-points kernel (about ten warp
// instructions per unit at 64 points, from instruction counts of one-type
// workloads), and of one event's product and sums.  A tile's warps take runs
// of events of equal summed work, not of equal dial count: the dial types
// differ in cost by up to ten times, and the warps of a tile wait for the
// slowest at the tile's barrier.  A tile's total stays below 2^16
// (kMaxTileDials * 40 + kMaxTileEvents * kEventCost).
GW_HD int dial_cost(int type, int n) {
  switch (type) {
    case kNorm: return 3;
    case kGrid: return 7;
    case kMonotonic:
    case kCompact:
    case kUniform: return 14;
    case kGeneral: return 19;
    case kGraph: return 15;
    case kBilinear: return 30;
    case kBicubic: return 40;
    case kTabulated: return 6;
    case kKriged: return 4 + (n < 31 ? n : 31);
    default: return 3;
  }
}
constexpr int kEventCost = 10;
static_assert(kMaxTileDials * 40 + kMaxTileEvents * kEventCost < 65536, "a tile's work must fit 16 bits");

// 16-bit per-event word: [0,10) first slot of the event, [10,13) local bin.
GW_HD uint16_t make_evinfo(int slot0, int lbin) {
  return (uint16_t)((slot0 & 0x3FF) | ((lbin & 0x7) << 10));
}
GW_HD int ev_slot(uint16_t v) { return v & 0x3FF; }
GW_HD int ev_lbin(uint16_t v) { return (v >> 10) & 0x7; }

struct TileDesc {
  uint64_t payload_off;   // byte offset of the tile payload (16-byte aligned)
  uint32_t dial0;         // first header of the tile
  uint32_t event0;        // first (bin-sorted) event of the tile
  uint32_t bin0;          // bin of the first event
  uint32_t slot0;         // partial-sum slot of (this tile, bin0)
  uint16_t ndials;
  uint16_t nevents;
  uint16_t payload_16b;   // payload size in 16-byte units
  uint16_t nbins;         // bin span: 1 + (last bin - bin0)
};
static_assert(sizeof(TileDesc) == 32, "TileDesc must stay 32 bytes");

// A knot grid shared by uniform-knot splines (the grid form): for every
// evaluated point k, the kernel that mirrors the parameters also forms
// xx = x[p0][k] * b + a (a = -low/step, b = 1/step in the engine precision),
// clamps it to [0, n - 1] when the parameter does not extrapolate, and stores
// the interval j = clamp(floor(xx), -1, n - 1) as the element offset of its
// coefficient block, 4 (j + 1), beside u = xx - j (GridPoint).
struct GridDesc {
  double a, b;
  int32_t p0;
  int32_t n;
  int32_t trunc;
  int32_t pad;
};
static_assert(sizeof(GridDesc) == 32, "GridDesc must stay 32 bytes");

// The interval of one grid at one point: u and the element offset of the
// coefficient block inside the dial's payload.
template <typename T>
struct alignas(sizeof(T) >= 8 ? 16 : 8) GridPoint {
  T u;
  int32_t jb;
};

// A table read by TABULATED / KRIGED dials.
struct TableDesc {
  int64_t offset;  // first element in the table arena
  int32_t size;    // entries per point
  int32_t per_k;   // 1: one copy per parameter point, laid out [entry][kpad]
  double lower;    // response clamp of the table's dials
  double upper;
};

// Device-side function that refills a table from fit parameters.
struct TableFn {
  int32_t table;
  int32_t kind;
  int32_t par[6];
  int64_t nodes;   // offset of the node energies in the node arena
};

}  // namespace gw
