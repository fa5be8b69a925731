// Time-step size without any device allocation: eif_decide_dt_noalloc.
//
// Who needs this. eif_decide_dt works on a context, and creating a context
// allocates device memory. Some callers cannot allocate: applications that
// hand every byte of device memory to their own pool and do not allow a
// library to call cudaMalloc behind their back, and time-critical loops in
// which a cudaMalloc or cudaFree would synchronise the whole device. This
// entry point computes the same time step (the reference's param_decide_dt)
// straight from the caller's device arrays, using only a fixed scratch array
// that lives in this library's static device memory.
//
// Scratch. g_noalloc_scratch below holds the column maxima of |ux|, the
// maximum of |uy| and a non-finite marker: EIF_NOALLOC_MAX_ITOT + 4 64-bit
// words (about 128 KiB) on
// every GPU that loads the library, kept until the process exits. Host code
// cannot use the symbol as a device address, so the address is looked up with
// cudaGetSymbolAddress once per device, on the first call made while that
// device is current; make that first call before any stream capture. Every
// call reuses the same array and clears it on the given stream before use, so
// calls that overlap on the GPU (on different streams, or from several host
// threads) race with each other and must be serialised by the caller.
#include "eif_internal.cuh"
#include <cfloat>
#include <mutex>

namespace {

__device__ __align__(256) unsigned long long g_noalloc_scratch[EIF_NOALLOC_MAX_ITOT + 4];

constexpr int NTX = 32, NTY = 8;
constexpr int MAX_DEVICES = 64;

// column maxima of |UX(i, j)| (i = 2..itot) and the maximum of |UY(i, j)| over
// rows 1..jtot, as bit patterns of non-negative doubles (ordered like the values);
// a NaN or an infinity among the values read sets *nonfinite
constexpr unsigned long long INF_BITS = 0x7ff0000000000000ull;
__global__ void k_noalloc_max(const double *__restrict__ ux, const double *__restrict__ uy, int ldx, int ldy, int itot,
                              int jtot, unsigned long long *__restrict__ colmax, unsigned long long *__restrict__ uymax,
                              unsigned long long *__restrict__ nonfinite) {
  const int i = 1 + blockIdx.x * NTX + threadIdx.x;
  unsigned long long mx = 0ull, my = 0ull;
  if (i <= itot) {
    for (int j = 1 + blockIdx.y * NTY + threadIdx.y; j <= jtot; j += NTY * gridDim.y) {
      if (i >= 2) {
        const unsigned long long b = __double_as_longlong(ux[(size_t)j * ldx + (i - 1)]) & 0x7fffffffffffffffull;
        mx = b > mx ? b : mx;
      }
      const unsigned long long b = __double_as_longlong(uy[(size_t)j * ldy + i]) & 0x7fffffffffffffffull;
      my = b > my ? b : my;
    }
  }
  if (mx >= INF_BITS || my >= INF_BITS) atomicOr(nonfinite, 1ull);
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(0xffffffffu, my, o);
    my = other > my ? other : my;
  }
  if (threadIdx.x == 0 && my) atomicMax(uymax, my);
  if (i >= 2 && i <= itot && mx) atomicMax(colmax + i, mx);
}

// x cell-centre spacing DXC(i) as set_coordinate forms it (src/param/init.c:117-139)
__device__ __forceinline__ double xf_of(int i, int itot, double dx) {
  return i == 1 ? 0. : (i == itot + 1 ? 1. : 1. * (i - 1) * dx);
}
__device__ __forceinline__ double xc_of(int i, int itot, double dx) {
  if (i == 0) return 0.;
  if (i == itot + 1) return 1.;
  return 0.5 * (xf_of(i, itot, dx) + xf_of(i + 1, itot, dx));
}

// dt from the maxima and the particle records (src/param/decide_dt.c:25-80)
__global__ void k_noalloc_final(const unsigned long long *__restrict__ colmax, const unsigned long long *__restrict__ uymax,
                                int itot, double dx, double dy, double Re, double sf_adv, double sf_dif, double sf_par,
                                const double *__restrict__ rec, int np, const unsigned long long *__restrict__ nonfinite,
                                double *__restrict__ dt_out) {
  const double small = 1.e-8;
  double dta = 5.e-2, dxmin = 1., dtp = DBL_MAX;
  for (int i = 2 + threadIdx.x; i <= itot; i += blockDim.x) {
    const double dxc = xc_of(i, itot, dx) - xc_of(i - 1, itot, dx);
    const double vel = fmax(__longlong_as_double((long long)colmax[i]), small);
    dta = fmin(dta, dxc / vel);
    dxmin = fmin(dxmin, dxc);
  }
  if (threadIdx.x == 0) dta = fmin(dta, dy / fmax(__longlong_as_double((long long)uymax[0]), small));
  const double delta = fmin(dx, dy);
  for (int n = threadIdx.x; n < np; n += blockDim.x) {
    const double *p = rec + (size_t)n * EIF_NFIELDS;
    const double r = fmax(p[EIF_P_A], p[EIF_P_B]);
    const double pux = fmax(fabs(p[EIF_P_UX]) + fabs(r * p[EIF_P_VZ]), small);
    const double puy = fmax(fabs(p[EIF_P_UY]) + fabs(r * p[EIF_P_VZ]), small);
    dtp = fmin(dtp, delta / fmax(pux, puy));
  }
  __shared__ double s[3][32];
  for (int o = 16; o > 0; o >>= 1) {
    dta = fmin(dta, __shfl_xor_sync(0xffffffffu, dta, o));
    dxmin = fmin(dxmin, __shfl_xor_sync(0xffffffffu, dxmin, o));
    dtp = fmin(dtp, __shfl_xor_sync(0xffffffffu, dtp, o));
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { s[0][w] = dta; s[1][w] = dxmin; s[2][w] = dtp; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); k++) {
      dta = fmin(dta, s[0][k]); dxmin = fmin(dxmin, s[1][k]); dtp = fmin(dtp, s[2][k]);
    }
    dta *= sf_adv;
    const double difx = 0.25 * Re * (dxmin * dxmin) * sf_dif;
    const double dify = 0.25 * Re * (dy * dy) * sf_dif;
    dtp *= sf_par;
    // a non-finite velocity gives no valid step: NaN, which no comparison accepts
    // (eif_decide_dt reports the same state as EIF_ERR_NONFINITE)
    *dt_out = *nonfinite ? __longlong_as_double(0x7ff8000000000000ll) : fmin(fmin(dta, fmin(difx, dify)), dtp);
  }
}

// device address of the scratch array, looked up once per device
std::mutex g_mutex;
unsigned long long *g_scratch_ptr[MAX_DEVICES] = {nullptr};

cudaError_t scratch_for_current_device(unsigned long long **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<unsigned long long *>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" int eif_decide_dt_noalloc(const double *ux, int ux_pitch, const double *uy, int uy_pitch, int itot,
                                     int jtot, double ly, double Re, const double *safefactors,
                                     const double *particles, int n_particles, double *dt, void *stream) {
  if (!ux || !uy || !dt || !safefactors || itot < 2 || jtot < 1 || !(ly > 0.) || !(Re > 0.) ||
      ux_pitch < itot + 1 || uy_pitch < itot + 2 || n_particles < 0 || (n_particles > 0 && !particles))
    return EIF_ERR_ARG;
  if (itot > EIF_NOALLOC_MAX_ITOT) return EIF_ERR_TOO_LARGE;
  unsigned long long *scratch = nullptr;
  if (scratch_for_current_device(&scratch) != cudaSuccess) return EIF_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned long long *colmax = scratch, *uymax = scratch + itot + 2, *nonfinite = scratch + itot + 3;
  // the array keeps the previous call's maxima and marker: clear what this call reads
  if (cudaMemsetAsync(scratch, 0, sizeof(unsigned long long) * (itot + 4), s) != cudaSuccess) return EIF_ERR_CUDA;
  int sms = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return EIF_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return EIF_ERR_CUDA;
  const int gx = (itot + NTX - 1) / NTX;
  int gy = (jtot + NTY - 1) / NTY;
  if (gx * gy > sms * 8) gy = (sms * 8 + gx - 1) / gx;
  if (gy < 1) gy = 1;
  k_noalloc_max<<<dim3(gx, gy), dim3(NTX, NTY), 0, s>>>(ux, uy, ux_pitch, uy_pitch, itot, jtot, colmax, uymax,
                                                         nonfinite);
  if (cudaGetLastError() != cudaSuccess) return EIF_ERR_CUDA;
  const double dx = 1. / itot, dy = ly / jtot;
  k_noalloc_final<<<1, 256, 0, s>>>(colmax, uymax, itot, dx, dy, Re, safefactors[0], safefactors[1], safefactors[2],
                                    particles, n_particles, nonfinite, dt);
  if (cudaGetLastError() != cudaSuccess) return EIF_ERR_CUDA;
  return EIF_OK;
}
