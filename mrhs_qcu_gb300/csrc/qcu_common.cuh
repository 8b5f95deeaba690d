// Shared device/host definitions of the GB300 MRHS Wilson library.
//
// Internal (device-resident) layouts:
//   gauge  [mu=4][parity=2][N*N][Vh] complex<P>   component-major per link,
//          the reference's "coalesced" gauge order
//          (include/basic_data/qcu_point.cuh:84-88 of the reference);
//   fermion MRHS field [4N][Vh][nrhs] complex<P>: component-major, RHS
//          innermost, so a warp reading one component for consecutive sites
//          reads one contiguous span; for 16-bit storage an FP32 scale per
//          (site, RHS) in a separate [Vh][nrhs] array, the stored values being
//          component / scale.
// P is FP64 (double2), FP32 (float2), FP16 (__half2) or BF16 (__nv_bfloat162).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <stdexcept>
#include <string>

namespace qcu {

// precision codes: the reference's QCU_PRECISION values (include/qcu_enum.h:4
// of the reference) plus BF16 as an extension, and BF16 in the site-major
// layout (below) as a storage code of its own
enum Prec : int { PREC_HALF = 0, PREC_SINGLE = 1, PREC_DOUBLE = 2, PREC_BF16 = 4, PREC_BF16S = 5 };

inline bool prec_valid(int p) {
  return p == PREC_HALF || p == PREC_SINGLE || p == PREC_DOUBLE || p == PREC_BF16 || p == PREC_BF16S;
}
inline bool prec_is16(int p) { return p == PREC_HALF || p == PREC_BF16 || p == PREC_BF16S; }
// BF16 storage of either layout
inline bool prec_bf16(int p) { return p == PREC_BF16 || p == PREC_BF16S; }
// Field layouts.  Component-major (every code but PREC_BF16S): component c of
// site s, RHS r at (c * Vh + s) * nrhs + r.  Site-major (PREC_BF16S): at
// (s * 4N + c) * nrhs + r, so one site's block of all components and RHS is
// one contiguous run (the tensor-core kernel copies it as one operand tile).
// Both keep the RHS innermost, so elementwise and per-RHS operations are
// layout-blind.
__host__ __device__ constexpr bool prec_site_major(int p) { return p == PREC_BF16S; }
// element strides (in complexes) between components and between sites
__host__ __device__ inline int64_t field_comp_stride(int p, int64_t vh, int ncomp, int nrhs) {
  return prec_site_major(p) ? (int64_t)nrhs : vh * nrhs;
}
__host__ __device__ inline int64_t field_site_stride(int p, int64_t vh, int ncomp, int nrhs) {
  return prec_site_major(p) ? (int64_t)ncomp * nrhs : (int64_t)nrhs + 0 * vh;
}
// FP16 fields carry a per-(site, RHS) FP32 scale; BF16 has the FP32 exponent
// range, so its fields are stored unscaled
inline bool prec_has_norm(int p) { return p == PREC_HALF; }
inline int prec_complex_bytes(int p) { return p == PREC_DOUBLE ? 16 : (p == PREC_SINGLE ? 8 : 4); }
inline const char* prec_name(int p) {
  switch (p) {
    case PREC_HALF: return "fp16";
    case PREC_SINGLE: return "fp32";
    case PREC_DOUBLE: return "fp64";
    case PREC_BF16: return "bf16";
    case PREC_BF16S: return "bf16-site";
  }
  return "?";
}

// error codes returned by the extended API and recorded for qcuGetLastError()
enum Status : int {
  QCU_OK = 0,
  QCU_ERR_NOT_INITIALIZED = 1,
  QCU_ERR_INVALID_ARGUMENT = 2,
  QCU_ERR_UNSUPPORTED = 3,
  QCU_ERR_CUDA = 4,
  QCU_ERR_NO_GAUGE = 5,
  QCU_ERR_NO_OPERATOR = 6,
  QCU_ERR_NOT_CONVERGED = 7,
  QCU_ERR_BREAKDOWN = 8,
  QCU_ERR_DEVICE_TIMEOUT = 9,
  QCU_ERR_OUT_OF_MEMORY = 10,
  QCU_ERR_CAPACITY = 11,
};

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define QCU_CHECK_CUDA(call)                                                                              \
  do {                                                                                                    \
    cudaError_t e_ = (call);                                                                              \
    if (e_ != cudaSuccess)                                                                                \
      throw ::qcu::Error(e_ == cudaErrorMemoryAllocation ? ::qcu::QCU_ERR_OUT_OF_MEMORY : ::qcu::QCU_ERR_CUDA, \
                         std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " + __FILE__ + ":" +    \
                             std::to_string(__LINE__));                                                   \
  } while (0)

#define QCU_REQUIRE(cond, code, msg)                     \
  do {                                                   \
    if (!(cond)) throw ::qcu::Error((code), (msg));      \
  } while (0)

// Host-side fault injection for the failure tests: when the environment
// variable QCU_INJECT_FAILURE names this site ("session": creating a session,
// "solver": creating a solver engine), a host allocation failure is raised
// there, which the C ABI reports as QCU_ERR_OUT_OF_MEMORY.
void inject_failure(const char* site);

// ---------------------------------------------------------------------------
// fast unsigned division by a runtime constant (round-up multiplier method):
// for d >= 1 and n < 2^31, q = umulhi(n, m) >> s with s = ceil(log2 d) and
// m = floor(2^(32+s) / d) + 1 (computed in 64 bits); exact for all n < 2^31.
struct FastDiv {
  uint32_t d, m, s;
  FastDiv() : d(1), m(0), s(0) {}
  explicit FastDiv(uint32_t div) : d(div) {
    s = 0;
    while ((1u << s) < d) s++;
    uint64_t one = 1;
    m = (d == 1) ? 0u : (uint32_t)(((one << (32 + s)) / d) + 1 - (one << 32));
    // m holds the low 32 bits of the 33-bit multiplier; see div() below
  }
  __host__ __device__ __forceinline__ uint32_t div(uint32_t n) const {
#ifdef __CUDA_ARCH__
    uint32_t hi = __umulhi(n, m);
#else
    uint32_t hi = (uint32_t)(((uint64_t)n * m) >> 32);
#endif
    // multiplier = 2^32 + m:  floor(n * (2^32 + m) / 2^(32+s)) = (n + hi) >> s
    return d == 1 ? n : (uint32_t)(((uint64_t)n + hi) >> s);
  }
  __host__ __device__ __forceinline__ void divmod(uint32_t n, uint32_t& q, uint32_t& r) const {
    q = div(n);
    r = n - q * d;
  }
};

// lattice geometry of one even-odd half lattice
struct Geometry {
  int L[4];      // X, Y, Z, T (full X extent)
  int hx;        // X / 2
  int vh;        // half volume
  int plane;     // hx * Ly
  int cube;      // hx * Ly * Lz
  FastDiv div_hx, div_y, div_z;
};

inline Geometry make_geometry(const int L[4]) {
  Geometry g;
  for (int i = 0; i < 4; i++) g.L[i] = L[i];
  g.hx = L[0] / 2;
  g.plane = g.hx * L[1];
  g.cube = g.plane * L[2];
  g.vh = g.cube * L[3];
  g.div_hx = FastDiv((uint32_t)g.hx);
  g.div_y = FastDiv((uint32_t)L[1]);
  g.div_z = FastDiv((uint32_t)L[2]);
  return g;
}

// Coordinates of even-odd site s (its index within one parity, x halved) and
// of its eight neighbours.  Hop d = 2 mu + (backward ? 1 : 0); p is the parity
// of the site's half-field.  An x neighbour of a site whose (y + z + t) parity
// eo differs from p sits at the same index or the next one (forward), at the
// previous one or the same (backward).
struct EoSite {
  uint32_t site, xh, y, z, t, eo;
  __host__ __device__ __forceinline__ EoSite(const Geometry& g, uint32_t s) : site(s) {
    uint32_t rest, rest2;
    g.div_hx.divmod(s, rest, xh);
    g.div_y.divmod(rest, rest2, y);
    g.div_z.divmod(rest2, t, z);
    eo = (y + z + t) & 1u;
  }
  __host__ __device__ __forceinline__ uint32_t nb(const Geometry& g, uint32_t p, int d) const {
    const uint32_t hx = (uint32_t)g.hx, ly = (uint32_t)g.L[1], lz = (uint32_t)g.L[2], lt = (uint32_t)g.L[3];
    const uint32_t plane = (uint32_t)g.plane, cube = (uint32_t)g.cube;
    switch (d) {
      case 0: return (eo != p) ? (xh == hx - 1 ? site - (hx - 1) : site + 1) : site;
      case 1: return (eo == p) ? (xh == 0 ? site + (hx - 1) : site - 1) : site;
      case 2: return (y == ly - 1) ? site - (ly - 1) * hx : site + hx;
      case 3: return (y == 0) ? site + (ly - 1) * hx : site - hx;
      case 4: return (z == lz - 1) ? site - (lz - 1) * plane : site + plane;
      case 5: return (z == 0) ? site + (lz - 1) * plane : site - plane;
      case 6: return (t == lt - 1) ? site - (lt - 1) * cube : site + cube;
      default: return (t == 0) ? site + (lt - 1) * cube : site - cube;
    }
  }
};

// ---------------------------------------------------------------------------
// storage traits: how a complex number of precision P sits in memory and how
// it converts to the compute type (double for FP64, float otherwise)
template <int P> struct Store;

template <> struct Store<PREC_DOUBLE> {
  using elem = double2;   // one complex
  using real = double;
  static constexpr bool has_norm = false;
  __device__ __forceinline__ static double2 to_c(double2 v) { return v; }
  __device__ __forceinline__ static double2 from_c(double2 v) { return v; }
};
template <> struct Store<PREC_SINGLE> {
  using elem = float2;
  using real = float;
  static constexpr bool has_norm = false;
  __device__ __forceinline__ static float2 to_c(float2 v) { return v; }
  __device__ __forceinline__ static float2 from_c(float2 v) { return v; }
};
template <> struct Store<PREC_HALF> {
  using elem = __half2;
  using real = float;
  static constexpr bool has_norm = true;
  __device__ __forceinline__ static float2 to_c(__half2 v) { return __half22float2(v); }
  __device__ __forceinline__ static __half2 from_c(float2 v) { return __float22half2_rn(v); }
};
template <> struct Store<PREC_BF16> {
  using elem = __nv_bfloat162;
  using real = float;
  static constexpr bool has_norm = false;
  __device__ __forceinline__ static float2 to_c(__nv_bfloat162 v) { return __bfloat1622float2(v); }
  __device__ __forceinline__ static __nv_bfloat162 from_c(float2 v) { return __float22bfloat162_rn(v); }
};
// site-major BF16: the same element, another layout
template <> struct Store<PREC_BF16S> : Store<PREC_BF16> {};

template <typename R> struct cplx;
template <> struct cplx<float> { using t = float2; };
template <> struct cplx<double> { using t = double2; };

}  // namespace qcu
