// C ABI of include/eif.h: context lifetime, state transfer, stage entry points
// and the time-step orchestration of integrate (src/main.c:13-55).
#include "eif_internal.cuh"
#include <cstdio>
#include <cstdarg>
#include <cstring>
#include <cstdlib>
#include <cmath>
#include <new>
#include <vector>

namespace eif {

int fail(eif_ctx *c, int code, const char *fmt, ...) {
  if (c) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof(c->err), fmt, ap);
    va_end(ap);
  }
  return code;
}

int check_cuda(eif_ctx *c, cudaError_t e, const char *what) {
  return fail(c, EIF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int launch_check(eif_ctx *c, const char *file, int line) {
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && c->sync_debug) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(c, EIF_ERR_CUDA, "kernel launched at %s:%d: %s", file, line, cudaGetErrorString(e));
  if (c->sync_debug) {
    int rc = check_records(c);
    if (rc) return fail(c, rc, "%s (after the kernel launched at %s:%d)", c->err, file, line);
  }
  return EIF_OK;
}

// read the bounds-guard record (after a synchronisation) and report it
int check_records(eif_ctx *c) {
  if (!c->d_check) return EIF_OK;
  EIF_CK(c, cudaMemcpyAsync(c->h_check, c->d_check, sizeof(unsigned long long) * 4, cudaMemcpyDeviceToHost, c->stream));
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  if (c->h_check[0] == 0ull) return EIF_OK;
  const unsigned long long tag = c->h_check[1], idx = c->h_check[2], bound = c->h_check[3];
  EIF_CK(c, cudaMemsetAsync(c->d_check, 0, sizeof(unsigned long long) * 4, c->stream));
  return fail(c, EIF_ERR_CUDA, "bounds guard %llu: index %llu outside [0, %llu)", tag, idx, bound);
}

// Particle-only work beside the fluid kernels. The kernels of a stage and their
// data dependences are unchanged; work that shares no buffer with the fluid kernels
// launched in between is moved to the side stream, which forks from the main stream
// and is joined back before the first kernel that needs its results. Off while the
// per-stage profiler or per-launch synchronisation is active.
bool overlap_on(const eif_ctx *c) { return c->side && !c->sync_debug && !c->prof.enabled; }

namespace {

// launches between begin and end go to the side stream, after the work already on the
// main stream; end records `ev` on the side stream and restores the main stream
struct SideScope {
  eif_ctx *c;
  bool active = false;
  explicit SideScope(eif_ctx *c_) : c(c_) {}
  int begin() {
    cudaError_t e = cudaEventRecord(c->ev_fork, c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->side, c->ev_fork, 0);
    if (e != cudaSuccess) return check_cuda(c, e, "fork to the side stream");
    c->main_stream = c->stream;
    c->stream = c->side;
    active = true;
    return EIF_OK;
  }
  // records ev on the side stream at this point of its work
  int mark(cudaEvent_t ev) {
    const cudaError_t e = cudaEventRecord(ev, c->side);
    return e == cudaSuccess ? EIF_OK : check_cuda(c, e, "cudaEventRecord (side stream)");
  }
  int end(cudaEvent_t ev) {
    if (!active) return EIF_OK;
    c->stream = c->main_stream;
    active = false;
    const cudaError_t e = cudaEventRecord(ev, c->side);
    return e == cudaSuccess ? EIF_OK : check_cuda(c, e, "cudaEventRecord (side stream)");
  }
  ~SideScope() {
    if (active) c->stream = c->main_stream;
  }
};

int join(eif_ctx *c, cudaEvent_t ev) {
  const cudaError_t e = cudaStreamWaitEvent(c->stream, ev, 0);
  return e == cudaSuccess ? EIF_OK : check_cuda(c, e, "join of the side stream");
}

}  // namespace

// the part of an RK stage before the particle sub-iterations (src/main.c:14-35)
int rk_stage_front(eif_ctx *c, int rk) {
  int rc;
  const bool ibm = c->np > 0;
  if ((rc = launch_reset_increments(c))) return rc;
  if (ibm && overlap_on(c)) {
    // side: inertia at X (reads the current velocity buffer, which the predictor
    // does not write) and the collision forces at X (particle fields only); main:
    // predictor, band lists, exchange, Poisson, projection
    SideScope side(c);
    if ((rc = side.begin())) return rc;
    if ((rc = launch_inertia(c, 0))) return rc;
    if ((rc = side.mark(c->ev_ibm))) return rc;
    if ((rc = launch_collision(c, 0))) return rc;
    if ((rc = side.end(c->ev_coll))) return rc;
    if ((rc = launch_predictor(c, rk))) return rc;
    if ((rc = join(c, c->ev_ibm))) return rc;
    // the band lists after the join: the side stream's chain (boxes, inertia) is the
    // longer of the two branches
    if ((rc = launch_band_lists(c))) return rc;
    if ((rc = launch_exchange(c))) return rc;
    if ((rc = launch_potential(c, rk, ibm))) return rc;
    if ((rc = launch_correct(c, rk, ibm, true))) return rc;
    return join(c, c->ev_coll);
  }
  if ((rc = launch_inertia(c, 0))) return rc;
  if ((rc = launch_predictor(c, rk))) return rc;
  if (ibm && (rc = launch_exchange(c))) return rc;
  if ((rc = launch_potential(c, rk, ibm))) return rc;
  if ((rc = launch_correct(c, rk, ibm, true))) return rc;
  return launch_collision(c, 0);
}

// one particle sub-iteration (src/main.c:36-39): inertia at X + dX and the
// collision forces (independent, the latter on the side stream), then increments
int sub_iteration(eif_ctx *c, int rk) {
  int rc;
  if (c->np > 0 && overlap_on(c)) {
    SideScope side(c);
    if ((rc = side.begin())) return rc;
    if ((rc = launch_collision(c, 1))) return rc;
    if ((rc = side.end(c->ev_coll))) return rc;
    if ((rc = launch_inertia(c, 1))) return rc;
    if ((rc = join(c, c->ev_coll))) return rc;
  } else {
    if ((rc = launch_inertia(c, 1))) return rc;
    if ((rc = launch_collision(c, 1))) return rc;
  }
  return launch_increment(c, rk);
}

}  // namespace eif

using namespace eif;

namespace eif_xfer {

// Transfers of page-locked host arrays. A kernel reads or writes the host array
// through its device mapping and converts between the host row pitch and the
// device pitch in the same pass: one streaming pass over the interconnect, faster
// than the copy engines' pitched copies (measured 208 vs 166 GB/s host to device,
// 192 vs 153 GB/s device to host on GB300). Pageable arrays use cudaMemcpy2DAsync.
// s (velocities of the mixed form, else null): the values rounded to float as well
__global__ void k_rows_in(const double *__restrict__ h, double *__restrict__ d, float *__restrict__ s, int w,
                          int rows, int ld) {
  const size_t n = (size_t)w * rows;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = t / (unsigned)w, col = t - r * w;
    const double v = h[t];
    d[r * ld + col] = v;
    if (s) s[r * ld + col] = eifd::d2f(v);
  }
}
__global__ void k_rows_out(const double *__restrict__ d, double *__restrict__ h, int w, int rows, int ld) {
  const size_t n = (size_t)w * rows;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = t / (unsigned)w, col = t - r * w;
    h[t] = d[r * ld + col];
  }
}
// particle records (n x EIF_NFIELDS, host) <-> structure of arrays (device, pcap per field);
// slots n .. pcap-1 are zeroed on the way in
__global__ void k_records_in(const double *__restrict__ rec, double *__restrict__ P, int n, int pcap) {
  const size_t total = (size_t)EIF_NFIELDS * pcap;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const int f = (int)(t / pcap), k = (int)(t - (size_t)f * pcap);
    P[t] = k < n ? rec[(size_t)k * EIF_NFIELDS + f] : 0.;
  }
}
__global__ void k_records_out(const double *__restrict__ P, double *__restrict__ rec, int n, int pcap) {
  const size_t total = (size_t)EIF_NFIELDS * n;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / EIF_NFIELDS), f = (int)(t - (size_t)k * EIF_NFIELDS);
    rec[t] = P[(size_t)f * pcap + k];
  }
}

// device address of a page-locked host array, or null for pageable memory
void *mapped(const void *host) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// shadow (velocities of the mixed form, else null): the float copy of dst, kept with it
int rows_in(eif_ctx *c, double *dst, const double *host, int w, int rows, float *shadow = nullptr) {
  if (const double *hd = static_cast<const double *>(mapped(host))) {
    k_rows_in<<<c->sms * 4, 512, 0, c->stream>>>(hd, dst, shadow, w, rows, c->ld);
    EIF_LAUNCH_CK(c);
    return EIF_OK;
  }
  EIF_CK(c, cudaMemcpy2DAsync(dst, sizeof(double) * c->ld, host, sizeof(double) * w, sizeof(double) * w, rows,
                              cudaMemcpyHostToDevice, c->stream));
  if (shadow) return launch_round_to_float(c, dst, shadow, c->nfield);
  return EIF_OK;
}

// engine: the DMA engines even for mapped memory (a copy beside running kernels, which
// the copy kernel would take SMs from)
int rows_out(eif_ctx *c, double *host, const double *src, int w, int rows, cudaStream_t stream = nullptr,
             bool engine = false) {
  if (!stream) stream = c->stream;
  if (double *hd = engine ? nullptr : static_cast<double *>(mapped(host))) {
    k_rows_out<<<c->sms * 4, 512, 0, stream>>>(src, hd, w, rows, c->ld);
    EIF_LAUNCH_CK(c);
    return EIF_OK;
  }
  EIF_CK(c, cudaMemcpy2DAsync(host, sizeof(double) * w, src, sizeof(double) * c->ld, sizeof(double) * w, rows,
                              cudaMemcpyDeviceToHost, stream));
  return EIF_OK;
}

}  // namespace eif_xfer

using eif_xfer::mapped;
using eif_xfer::rows_in;
using eif_xfer::rows_out;

namespace {

// grid metrics exactly as set_coordinate computes them (src/param/init.c:105-167)
void host_metrics(eif_ctx *c) {
  const int itot = c->itot, jtot = c->jtot;
  c->h_xf = new double[itot + 2];
  c->h_xc = new double[itot + 2];
  c->h_dxf = new double[itot + 2];
  c->h_dxc = new double[itot + 2];
  c->h_yf = new double[jtot + 2];
  c->h_yc = new double[jtot + 2];
  // 0-based storage of XF(1..itot+1), XC(0..itot+1), DXF(1..itot), DXC(1..itot+1), YF(1..), YC(1..)
  const double dx = c->lx / itot;
  c->dx = dx;
  for (int i = 1; i <= itot + 1; i++) c->h_xf[i - 1] = 1. * (i - 1) * dx;
  c->h_xf[0] = 0.;
  c->h_xf[itot] = c->lx;
  for (int i = 1; i <= itot; i++) c->h_dxf[i - 1] = c->h_xf[i] - c->h_xf[i - 1];
  c->h_xc[0] = c->h_xf[0];
  for (int i = 1; i <= itot; i++) c->h_xc[i] = 0.5 * (c->h_xf[i - 1] + c->h_xf[i]);
  c->h_xc[itot + 1] = c->h_xf[itot];
  for (int i = 1; i <= itot + 1; i++) c->h_dxc[i - 1] = c->h_xc[i] - c->h_xc[i - 1];
  const double dy = c->ly / jtot;
  c->dy = dy;
  for (int j = 1; j <= jtot + 1; j++) c->h_yf[j - 1] = 0. + 1. * (j - 1) * dy;
  for (int j = 1; j <= jtot; j++) c->h_yc[j - 1] = 0. + 0.5 * (2 * j - 1) * dy;
}

int upload(eif_ctx *c, double **dst, const std::vector<double> &v) {
  EIF_CK(c, cudaMalloc((void **)dst, sizeof(double) * v.size()));
  EIF_CK(c, cudaMemcpy(*dst, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice));
  return EIF_OK;
}

int device_metrics(eif_ctx *c) {
  const int itot = c->itot, jtot = c->jtot;
  auto DXF = [&](int i) { return c->h_dxf[i - 1]; };
  auto DXC = [&](int i) { return c->h_dxc[i - 1]; };
  std::vector<double> xc(itot + 2), yc(jtot + 2, 0.), rdxf(itot + 2, 0.), rdxc(itot + 2, 0.), dxc(itot + 2, 0.);
  std::vector<double> cxm(itot + 2, 0.), cxp(itot + 2, 0.), cym(itot + 2, 0.), cyp(itot + 2, 0.);
  for (int i = 0; i <= itot + 1; i++) xc[i] = c->h_xc[i];
  for (int j = 1; j <= jtot; j++) yc[j] = c->h_yc[j - 1];
  for (int i = 1; i <= itot; i++) rdxf[i] = 1. / DXF(i);
  for (int i = 1; i <= itot + 1; i++) { rdxc[i] = 1. / DXC(i); dxc[i] = DXC(i); }
  for (int i = 2; i <= itot; i++) {
    // update_velocity.c:38-39
    cxm[i] = DXF(i - 1) / (2. * DXC(i));
    cxp[i] = DXF(i) / (2. * DXC(i));
  }
  for (int i = 1; i <= itot; i++) {
    // update_velocity.c:121-122
    cym[i] = DXC(i) / (2. * DXF(i));
    cyp[i] = DXC(i + 1) / (2. * DXF(i));
  }
  int rc;
  auto upload_f = [&](float **dst, const std::vector<double> &v) -> int {
    std::vector<float> f(v.begin(), v.end());
    EIF_CK(c, cudaMalloc((void **)dst, sizeof(float) * f.size()));
    EIF_CK(c, cudaMemcpy(*dst, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice));
    return EIF_OK;
  };
  if ((rc = upload_f(&c->rdxf_f, rdxf))) return rc;
  if ((rc = upload_f(&c->rdxc_f, rdxc))) return rc;
  {
    std::vector<float2> df(rdxc.size());
    for (size_t q = 0; q < rdxc.size(); q++) {
      const float hi = (float)rdxc[q];
      df[q] = make_float2(hi, (float)(rdxc[q] - (double)hi));
    }
    EIF_CK(c, cudaMalloc((void **)&c->rdxc_df, sizeof(float2) * df.size()));
    EIF_CK(c, cudaMemcpy(c->rdxc_df, df.data(), sizeof(float2) * df.size(), cudaMemcpyHostToDevice));
  }
  if ((rc = upload_f(&c->cxm_f, cxm))) return rc;
  if ((rc = upload_f(&c->cxp_f, cxp))) return rc;
  if ((rc = upload_f(&c->cym_f, cym))) return rc;
  if ((rc = upload_f(&c->cyp_f, cyp))) return rc;
  {
    // the mixed predictor's x metrics as floats are one value each away from the walls:
    // rdxf(1..itot), rdxc(2..itot), cxm and cxp (2..itot), cym (2..itot), cyp (1..itot-1);
    // only rdxc(1), cym(1) (cell 1) and rdxc(itot+1), cyp(itot) (cell itot) see the half
    // cells at the walls. Checked bitwise, so that the arguments give the loads' values.
    eif_ctx::UniformX u;
    u.rdxf = (float)rdxf[1];
    u.rdxc = (float)rdxc[2];
    u.cx = (float)cxm[2];
    u.cy = (float)cym[2];
    bool ok = itot >= 3 && !std::getenv("EIF_NO_UNIFORM_X");
    for (int i = 1; ok && i <= itot; i++) {
      ok = (float)rdxf[i] == u.rdxf;
      if (ok && i >= 2) ok = (float)rdxc[i] == u.rdxc && (float)cxm[i] == u.cx && (float)cxp[i] == u.cx &&
                             (float)cym[i] == u.cy;
      if (ok && i <= itot - 1) ok = (float)cyp[i] == u.cy;
    }
    u.on = ok;
    c->uni_x = u;
  }
  if ((rc = upload(c, &c->xc, xc))) return rc;
  if ((rc = upload(c, &c->yc, yc))) return rc;
  if ((rc = upload(c, &c->rdxf, rdxf))) return rc;
  if ((rc = upload(c, &c->rdxc, rdxc))) return rc;
  if ((rc = upload(c, &c->dxc, dxc))) return rc;
  {
    std::vector<double> dxf(itot + 2, 0.);
    for (int i = 1; i <= itot; i++) dxf[i] = DXF(i);
    if ((rc = upload(c, &c->dxf, dxf))) return rc;
  }
  if ((rc = upload(c, &c->cxm, cxm))) return rc;
  if ((rc = upload(c, &c->cxp, cxp))) return rc;
  if ((rc = upload(c, &c->cym, cym))) return rc;
  if ((rc = upload(c, &c->cyp, cyp))) return rc;
  return EIF_OK;
}

}  // namespace

namespace eif {
int check_flags(eif_ctx *c) {
  // called after a synchronisation; reports and clears kernel error flags
  unsigned f = *c->h_flags;
  if (f == 0u) return EIF_OK;
  *c->h_flags = 0u;
  EIF_CK(c, cudaMemsetAsync(c->d_flags, 0, sizeof(unsigned), c->stream));
  if (f & EIF_FLAG_NONFINITE) {
    c->src_nonfinite = true;
    return fail(c, EIF_ERR_NONFINITE, "non-finite velocity detected");
  }
  if (f & EIF_FLAG_NOCONV)
    return fail(c, EIF_ERR_NOCONV, "an iteration cap or a device list capacity was reached on the device");
  if (f & EIF_FLAG_TIMEOUT)
    return fail(c, EIF_ERR_CUDA, "a bounded wait on the device (a tile copy or a grid barrier) gave up");
  return EIF_OK;
}
}  // namespace eif

namespace {

// copy the scalars and flags to the host and wait
int sync_scalars(eif_ctx *c) {
  EIF_CK(c, cudaMemcpyAsync(c->h_scal, c->d_scal, sizeof(double) * 4, cudaMemcpyDeviceToHost, c->stream));
  EIF_CK(c, cudaMemcpyAsync(c->h_flags, c->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  c->dt_host = c->h_scal[0];
  int rc = check_records(c);
  if (rc) return rc;
  return check_flags(c);
}

int ensure_pcap(eif_ctx *c, int n) {
  if (n <= c->pcap && c->P) return EIF_OK;
  if (c->P) cudaFree(c->P);
  c->P = nullptr;
  const int cap = n > 0 ? n : 1;
  EIF_CK(c, cudaMalloc((void **)&c->P, sizeof(double) * EIF_NFIELDS * (size_t)cap));
  EIF_CK(c, cudaMemset(c->P, 0, sizeof(double) * EIF_NFIELDS * (size_t)cap));
  c->pcap = cap;
  return EIF_OK;
}

bool valid_rk(int rk) { return rk >= 0 && rk < 3; }

// one RK stage of integrate (src/main.c:14-53); *sub receives the sub-iterations
int rk_stage(eif_ctx *c, int rk, int *sub) {
  int rc;
  if ((rc = rk_stage_front(c, rk))) return rc;
  int s = 0;
  for (s = 0;; s++) {
    if ((rc = sub_iteration(c, rk))) return rc;
    if ((rc = sync_scalars(c))) return rc;
    if (c->h_scal[1] < 1.e-8) break;
    if (s > 100) break;
  }
  if (sub) *sub = s + 1;
  return launch_update_particles(c);
}

}  // namespace

extern "C" {

int eif_create(const eif_config_t *cfg, eif_ctx **out) {
  if (!cfg || !out) return EIF_ERR_ARG;
  *out = nullptr;
  eif_ctx *c = new (std::nothrow) eif_ctx();
  if (!c) return EIF_ERR_NOMEM;
  c->cfg = *cfg;
  if (cfg->itot < 4 || cfg->jtot < 3 || !(cfg->ly > 0.) || !(cfg->Re > 0.) ||
      (cfg->precision != EIF_PREC_FP64 && cfg->precision != EIF_PREC_MIXED)) {
    int rc = fail(c, EIF_ERR_ARG, "invalid configuration");
    delete c;
    return rc;
  }
  c->itot = cfg->itot;
  c->jtot = cfg->jtot;
  c->lx = 1.;
  c->ly = cfg->ly;
  c->ld = ((cfg->itot + 2) + 31) / 32 * 32;
  c->nfield = (size_t)c->ld * (c->jtot + 2);
  c->device = cfg->device;
  *out = c;
#define CK_CREATE(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return check_cuda(c, e_, #call); } while (0)
  CK_CREATE(cudaSetDevice(c->device));
  int sms = 0;
  CK_CREATE(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  c->sms = sms;
  CK_CREATE(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CK_CREATE(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
  CK_CREATE(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
  CK_CREATE(cudaEventCreateWithFlags(&c->ev_ibm, cudaEventDisableTiming));
  CK_CREATE(cudaEventCreateWithFlags(&c->ev_coll, cudaEventDisableTiming));
  CK_CREATE(cudaEventCreateWithFlags(&c->ev_fields, cudaEventDisableTiming));
  CK_CREATE(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
  host_metrics(c);
  int rc = device_metrics(c);
  if (rc) return rc;
  double **fields[] = {&c->ux[0], &c->ux[1], &c->uy[0], &c->uy[1], &c->p, &c->psi,
                       &c->sxa[0], &c->sxa[1], &c->sya[0], &c->sya[1], &c->dux, &c->duy, &c->qhat};
  for (double **f : fields) {
    CK_CREATE(cudaMalloc((void **)f, sizeof(double) * c->nfield));
    CK_CREATE(cudaMemset(*f, 0, sizeof(double) * c->nfield));
  }
  if (cfg->precision == EIF_PREC_MIXED) {
    float **ffields[] = {&c->sxf[0], &c->sxf[1], &c->syf[0], &c->syf[1], &c->uxf[0], &c->uxf[1], &c->uyf[0],
                         &c->uyf[1]};
    for (float **f : ffields) {
      CK_CREATE(cudaMalloc((void **)f, sizeof(float) * c->nfield));
      CK_CREATE(cudaMemset(*f, 0, sizeof(float) * c->nfield));
    }
  }
  CK_CREATE(cudaMalloc((void **)&c->d_coef, sizeof(float) * 32));
  CK_CREATE(cudaMemset(c->d_coef, 0, sizeof(float) * 32));
  CK_CREATE(cudaMalloc((void **)&c->d_scal, sizeof(double) * 4));
  CK_CREATE(cudaMemset(c->d_scal, 0, sizeof(double) * 4));
  CK_CREATE(cudaMalloc((void **)&c->d_inc, sizeof(unsigned long long) * 6));
  CK_CREATE(cudaMemset(c->d_inc, 0, sizeof(unsigned long long) * 6));
  CK_CREATE(cudaMalloc((void **)&c->d_flags, sizeof(unsigned)));
  CK_CREATE(cudaMemset(c->d_flags, 0, sizeof(unsigned)));
  CK_CREATE(cudaMallocHost((void **)&c->h_scal, sizeof(double) * 4));
  CK_CREATE(cudaMallocHost((void **)&c->h_flags, sizeof(unsigned)));
  *c->h_flags = 0u;
  CK_CREATE(cudaMallocHost((void **)&c->h_check, sizeof(unsigned long long) * 4));
  CK_CREATE(cudaMallocHost((void **)&c->h_slots, sizeof(eif_ctx::StepSlot) * 2));
  for (auto &e : c->ev_step) CK_CREATE(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  CK_CREATE(cudaMalloc((void **)&c->d_check, sizeof(unsigned long long) * 4));
  CK_CREATE(cudaMemset(c->d_check, 0, sizeof(unsigned long long) * 4));
  c->sync_debug = getenv("EIF_SYNC_DEBUG") != nullptr;
  c->use_graphs = getenv("EIF_NO_GRAPHS") == nullptr;
  c->memo_on = getenv("EIF_NO_MEMO") == nullptr;
#undef CK_CREATE
  rc = poisson_init(c);
  if (rc) return rc;
  if ((rc = predictor_prepare(c))) return rc;
  rc = ensure_pcap(c, 1);
  if (rc) return rc;
  rc = launch_boundaries(c);
  if (rc) return rc;
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  return EIF_OK;
}

int eif_destroy(eif_ctx *c) {
  if (!c) return EIF_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->adj) eif_adjoint_end(c);
  snapshot_free(c);
  stats_free(c);
  double *ptrs[] = {c->ux[0], c->ux[1], c->uy[0], c->uy[1], c->p, c->psi, c->sxa[0], c->sxa[1], c->sya[0],
                    c->sya[1], c->dux, c->duy, c->qhat, c->xc, c->yc, c->rdxf, c->rdxc, c->cxm, c->cxp, c->cym,
                    c->cyp, c->dxc, c->dxf, c->P, c->d_scal};
  for (double *p : ptrs) if (p) cudaFree(p);
  if (c->d_coef) cudaFree(c->d_coef);
  if (c->rdxc_df) cudaFree(c->rdxc_df);
  if (c->d_inc) cudaFree(c->d_inc);
  graphs_free(c);
  float *fptrs[] = {c->rdxf_f, c->rdxc_f, c->cxm_f, c->cxp_f, c->cym_f, c->cyp_f, c->sxf[0], c->sxf[1], c->syf[0],
                    c->syf[1], c->uxf[0], c->uxf[1], c->uyf[0], c->uyf[1]};
  for (float *p : fptrs) if (p) cudaFree(p);
  if (c->d_flags) cudaFree(c->d_flags);
  if (c->d_check) cudaFree(c->d_check);
  if (c->h_check) cudaFreeHost(c->h_check);
  if (c->h_slots) cudaFreeHost(c->h_slots);
  for (auto &e : c->ev_step)
    if (e) cudaEventDestroy(e);
  if (c->h_scal) cudaFreeHost(c->h_scal);
  if (c->h_flags) cudaFreeHost(c->h_flags);
  poisson_free(c);
  ibm_free(c);
  profile_free(c);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_ibm) cudaEventDestroy(c->ev_ibm);
  if (c->ev_coll) cudaEventDestroy(c->ev_coll);
  if (c->ev_fields) cudaEventDestroy(c->ev_fields);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete[] c->h_xf; delete[] c->h_xc; delete[] c->h_dxf; delete[] c->h_dxc; delete[] c->h_yf; delete[] c->h_yc;
  delete c;
  return EIF_OK;
}

const char *eif_last_error(const eif_ctx *c) { return c ? c->err : "null context"; }

int eif_synchronize(eif_ctx *c) {
  if (!c) return EIF_ERR_ARG;
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  return EIF_OK;
}

void *eif_stream(eif_ctx *c) { return c ? (void *)c->stream : nullptr; }

int eif_push_fluid(eif_ctx *c, const double *ux, const double *uy, const double *p) {
  if (!c || !ux || !uy || !p) return EIF_ERR_ARG;
  const int rows = c->jtot + 2;
  int rc;
  if ((rc = rows_in(c, c->ux[c->cur], ux, c->itot + 1, rows, c->uxf[c->cur]))) return rc;
  if ((rc = rows_in(c, c->uy[c->cur], uy, c->itot + 2, rows, c->uyf[c->cur]))) return rc;
  if ((rc = rows_in(c, c->p, p, c->itot + 2, rows))) return rc;
  if (c->src_nonfinite) {
    for (double *f : {c->sxa[0], c->sxa[1], c->sya[0], c->sya[1]})
      EIF_CK(c, cudaMemsetAsync(f, 0, sizeof(double) * c->nfield, c->stream));
    if (c->cfg.precision == EIF_PREC_MIXED)
      for (float *f : {c->sxf[0], c->sxf[1], c->syf[0], c->syf[1]})
        EIF_CK(c, cudaMemsetAsync(f, 0, sizeof(float) * c->nfield, c->stream));
    c->src_nonfinite = false;
  }
  rc = launch_boundaries(c);
  if (rc) return rc;
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  c->fluid_pushed = true;
  return EIF_OK;
}

int eif_pull_fluid(eif_ctx *c, double *ux, double *uy, double *p, double *psi) {
  if (!c) return EIF_ERR_ARG;
  const int rows = c->jtot + 2;
  int rc;
  if (ux && (rc = rows_out(c, ux, c->ux[c->cur], c->itot + 1, rows))) return rc;
  if (uy && (rc = rows_out(c, uy, c->uy[c->cur], c->itot + 2, rows))) return rc;
  if (p && (rc = rows_out(c, p, c->p, c->itot + 2, rows))) return rc;
  if (psi) {
    // psi in double: the field itself, or psi1 + psi2 of the refined solve widened in scratch
    const double *src = c->psi;
    if (c->psi_pair) {
      if ((rc = launch_psi_to_double(c, c->qhat))) return rc;
      src = c->qhat;
    }
    if ((rc = rows_out(c, psi, src, c->itot + 2, rows))) return rc;
  }
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  return check_records(c);
}

int eif_push_particles(eif_ctx *c, int n, const double *rec) {
  if (!c || n < 0 || (n > 0 && !rec)) return EIF_ERR_ARG;
  // The IBM buffers, and the step graphs that hold them, are kept when the particle
  // count is unchanged and the buffers already cover the pushed radii (a driver that
  // re-pushes the state every step); otherwise they are rebuilt.
  const size_t chunks = ibm_tasks_needed(c, rec, n);
  const bool reuse = c->P && n == c->np && n <= c->pcap && (n == 0 || (c->box && chunks <= (size_t)c->chunk_cap));
  if (!reuse) {
    graphs_free(c);
    c->buf_gen++;
    int rc = ensure_pcap(c, n);
    if (rc) return rc;
  }
  c->incr_zero = false;
  c->boxes_x_valid = false;
  c->weights_x_valid = false;
  if (const double *rd = n > 0 ? static_cast<const double *>(mapped(rec)) : nullptr) {
    eif_xfer::k_records_in<<<c->sms, 256, 0, c->stream>>>(rd, c->P, n, c->pcap);
    EIF_LAUNCH_CK(c);
    EIF_CK(c, cudaStreamSynchronize(c->stream));
  } else {
    std::vector<double> soa((size_t)EIF_NFIELDS * c->pcap, 0.);
    for (int f = 0; f < EIF_NFIELDS; f++)
      for (int k = 0; k < n; k++) soa[(size_t)f * c->pcap + k] = rec[(size_t)k * EIF_NFIELDS + f];
    EIF_CK(c, cudaStreamSynchronize(c->stream));
    EIF_CK(c, cudaMemcpy(c->P, soa.data(), sizeof(double) * soa.size(), cudaMemcpyHostToDevice));
  }
  c->np = n;
  return reuse ? EIF_OK : ibm_reserve(c, chunks);
}

int eif_pull_particles(eif_ctx *c, int n, double *rec) {
  if (!c || n != c->np || (n > 0 && !rec)) return fail(c, EIF_ERR_ARG, "particle count mismatch (%d vs %d)", n, c ? c->np : 0);
  if (n == 0) return EIF_OK;
  if (double *rd = static_cast<double *>(mapped(rec))) {
    eif_xfer::k_records_out<<<c->sms, 256, 0, c->stream>>>(c->P, rd, n, c->pcap);
    EIF_LAUNCH_CK(c);
    EIF_CK(c, cudaStreamSynchronize(c->stream));
    return check_records(c);
  }
  std::vector<double> soa((size_t)EIF_NFIELDS * c->pcap);
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  EIF_CK(c, cudaMemcpy(soa.data(), c->P, sizeof(double) * soa.size(), cudaMemcpyDeviceToHost));
  for (int f = 0; f < EIF_NFIELDS; f++)
    for (int k = 0; k < n; k++) rec[(size_t)k * EIF_NFIELDS + f] = soa[(size_t)f * c->pcap + k];
  return check_records(c);
}

// source arrays: SRCUXA(i,j) for i=2..itot at ux index, SRCUYA(i,j) for i=1..itot at uy index
int eif_pull_src(eif_ctx *c, double *uxa, double *uxb, double *uya, double *uyb) {
  if (!c) return EIF_ERR_ARG;
  const size_t dp = sizeof(double) * c->ld;
  const size_t wx = sizeof(double) * (c->itot - 1), wy = sizeof(double) * c->itot;
  const int a = c->scur, b = 1 - c->scur;
  if (c->cfg.precision == EIF_PREC_MIXED) {
    // the mixed form keeps these terms in float: widen each through the scratch field
    const float *srcs[4] = {c->sxf[a], c->sxf[b], c->syf[a], c->syf[b]};
    double *dsts[4] = {uxa, uxb, uya, uyb};
    for (int k = 0; k < 4; k++) {
      if (!dsts[k]) continue;
      int rc = launch_f2d_copy(c, srcs[k], c->qhat, c->nfield);
      if (rc) return rc;
      const size_t w = k < 2 ? wx : wy;
      EIF_CK(c, cudaMemcpy2DAsync(dsts[k], w, c->qhat + c->ld + 1, dp, w, c->jtot, cudaMemcpyDeviceToHost, c->stream));
      EIF_CK(c, cudaStreamSynchronize(c->stream));
    }
    return check_records(c);
  }
  // SRCUXA(2,1) sits at ux index (2,1) -> row 1, column 1
  if (uxa) EIF_CK(c, cudaMemcpy2DAsync(uxa, wx, c->sxa[a] + c->ld + 1, dp, wx, c->jtot, cudaMemcpyDeviceToHost, c->stream));
  if (uxb) EIF_CK(c, cudaMemcpy2DAsync(uxb, wx, c->sxa[b] + c->ld + 1, dp, wx, c->jtot, cudaMemcpyDeviceToHost, c->stream));
  if (uya) EIF_CK(c, cudaMemcpy2DAsync(uya, wy, c->sya[a] + c->ld + 1, dp, wy, c->jtot, cudaMemcpyDeviceToHost, c->stream));
  if (uyb) EIF_CK(c, cudaMemcpy2DAsync(uyb, wy, c->sya[b] + c->ld + 1, dp, wy, c->jtot, cudaMemcpyDeviceToHost, c->stream));
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  return check_records(c);
}

int eif_push_src(eif_ctx *c, const double *uxa, const double *uya) {
  if (!c || !uxa || !uya) return EIF_ERR_ARG;
  const size_t dp = sizeof(double) * c->ld;
  const size_t wx = sizeof(double) * (c->itot - 1), wy = sizeof(double) * c->itot;
  if (c->cfg.precision == EIF_PREC_MIXED) {
    float *dsts[2] = {c->sxf[c->scur], c->syf[c->scur]};
    const double *srcs[2] = {uxa, uya};
    for (int k = 0; k < 2; k++) {
      EIF_CK(c, cudaMemsetAsync(c->qhat, 0, sizeof(double) * c->nfield, c->stream));
      const size_t w = k == 0 ? wx : wy;
      EIF_CK(c, cudaMemcpy2DAsync(c->qhat + c->ld + 1, dp, srcs[k], w, w, c->jtot, cudaMemcpyHostToDevice, c->stream));
      int rc = launch_d2f_copy(c, c->qhat, dsts[k], c->nfield);
      if (rc) return rc;
    }
    EIF_CK(c, cudaStreamSynchronize(c->stream));
    return EIF_OK;
  }
  EIF_CK(c, cudaMemcpy2DAsync(c->sxa[c->scur] + c->ld + 1, dp, uxa, wx, wx, c->jtot, cudaMemcpyHostToDevice, c->stream));
  EIF_CK(c, cudaMemcpy2DAsync(c->sya[c->scur] + c->ld + 1, dp, uya, wy, wy, c->jtot, cudaMemcpyHostToDevice, c->stream));
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  return EIF_OK;
}

int eif_pull_ibm_fields(eif_ctx *c, double *dux, double *duy) {
  if (!c || !dux || !duy) return EIF_ERR_ARG;
  const size_t dp = sizeof(double) * c->ld, wy = sizeof(double) * (c->itot + 2);
  if (c->cfg.precision == EIF_PREC_MIXED) {
    // the mixed form keeps the field response in single precision: widen it in scratch
    double *dst[2] = {dux, duy};
    const float *src[2] = {reinterpret_cast<const float *>(c->dux), reinterpret_cast<const float *>(c->duy)};
    for (int k = 0; k < 2; k++) {
      int rc = launch_f2d_copy(c, src[k], c->qhat, c->nfield);
      if (rc) return rc;
      EIF_CK(c, cudaMemcpy2DAsync(dst[k], wy, c->qhat, dp, wy, c->jtot + 2, cudaMemcpyDeviceToHost, c->stream));
      EIF_CK(c, cudaStreamSynchronize(c->stream));
    }
    return check_records(c);
  }
  EIF_CK(c, cudaMemcpy2DAsync(dux, wy, c->dux, dp, wy, c->jtot + 2, cudaMemcpyDeviceToHost, c->stream));
  EIF_CK(c, cudaMemcpy2DAsync(duy, wy, c->duy, dp, wy, c->jtot + 2, cudaMemcpyDeviceToHost, c->stream));
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  return check_records(c);
}

int eif_decide_dt(eif_ctx *c, double *dt) {
  if (!c) return EIF_ERR_ARG;
  int rc = launch_decide_dt(c);
  if (rc) return rc;
  if (dt) {
    if ((rc = sync_scalars(c))) return rc;
    *dt = c->dt_host;
  }
  return EIF_OK;
}

int eif_set_dt(eif_ctx *c, double dt) {
  if (!c || !(dt > 0.)) return EIF_ERR_ARG;
  c->h_scal[0] = dt;
  EIF_CK(c, cudaMemcpyAsync(c->d_scal, c->h_scal, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  int rc = launch_coef(c);
  if (rc) return rc;
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  c->dt_host = dt;
  return EIF_OK;
}

int eif_get_dt(eif_ctx *c, double *dt) {
  if (!c || !dt) return EIF_ERR_ARG;
  int rc = sync_scalars(c);
  if (rc) return rc;
  *dt = c->dt_host;
  return EIF_OK;
}

int eif_integrate(eif_ctx *c, int *substeps) {
  if (!c) return EIF_ERR_ARG;
  if (!c->fluid_pushed) return fail(c, EIF_ERR_STATE, "push the fluid state before integrating");
  if (int rc = tune_tiles(c)) return rc;
  for (int rk = 0; rk < 3; rk++) {
    int sub = 0;
    int rc = rk_stage(c, rk, &sub);
    if (rc) return rc;
    if (substeps) substeps[rk] = sub;
  }
  return sync_scalars(c);
}

namespace {

// host arrays that eif_advance_pull fills with the fields after the last step
struct FieldTargets {
  double *ux, *uy, *p;
};

int advance(eif_ctx *c, int nsteps, const FieldTargets *ft) {
  if (!c || nsteps < 0) return EIF_ERR_ARG;
  if (!c->fluid_pushed) return fail(c, EIF_ERR_STATE, "push the fluid state before integrating");
  if (int rc = tune_tiles(c)) return rc;
  bool fields_queued = false;
  if (c->use_graphs && !c->sync_debug && !c->prof.enabled) {
    // one graph launch per step (see graph.cu), queued one step ahead: step s + 1 is
    // launched before the host waits for the copies of step s's dt, flags and bounds
    // record, so the GPU does not idle between steps. When step s reports an error,
    // step s + 1 has already run on the device: it is waited for and counted too, so
    // that the step counter and time always describe the device state.
    auto finish = [&](int s) -> int {
      eif_ctx::StepSlot &h = c->h_slots[s & 1];
      EIF_CK(c, cudaEventSynchronize(c->ev_step[s & 1]));
      for (int k = 0; k < 4; k++) c->h_scal[k] = h.scal[k];
      c->dt_host = h.scal[0];
      c->step += 1;
      c->time += c->dt_host;
      if (h.check[0] != 0ull) {
        for (int k = 0; k < 4; k++) c->h_check[k] = h.check[k];
        EIF_CK(c, cudaStreamSynchronize(c->stream));
        EIF_CK(c, cudaMemsetAsync(c->d_check, 0, sizeof(unsigned long long) * 4, c->stream));
        return fail(c, EIF_ERR_CUDA, "bounds guard %llu: index %llu outside [0, %llu)", h.check[1], h.check[2],
                    h.check[3]);
      }
      if (h.flags != 0u) {
        EIF_CK(c, cudaStreamSynchronize(c->stream));
        *c->h_flags = h.flags;
        return check_flags(c);
      }
      return EIF_OK;
    };
    for (int s = 0; s < nsteps; s++) {
      int rc = step_graph_launch(c);
      if (rc) return rc;
      eif_ctx::StepSlot &h = c->h_slots[s & 1];
      EIF_CK(c, cudaMemcpyAsync(h.scal, c->d_scal, sizeof(double) * 4, cudaMemcpyDeviceToHost, c->stream));
      EIF_CK(c, cudaMemcpyAsync(&h.flags, c->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
      if (c->d_check) {
        EIF_CK(c, cudaMemcpyAsync(h.check, c->d_check, sizeof(unsigned long long) * 4, cudaMemcpyDeviceToHost,
                                  c->stream));
      } else {
        h.check[0] = 0ull;
      }
      EIF_CK(c, cudaEventRecord(c->ev_step[s & 1], c->stream));
      if (ft && s == nsteps - 1) {
        // the fields are final once the graph has recorded ev_fields (after the last
        // stage's projection): the first of them is copied on the DMA engines beside that
        // stage's particle work, which keeps the SMs; the others by the copy kernel (the
        // faster copy) once the step is done
        EIF_CK(c, cudaStreamWaitEvent(c->copy_stream, c->ev_fields, 0));
        const int rows = c->jtot + 2;
        double *hosts[3] = {ft->ux, ft->uy, ft->p};
        const double *srcs[3] = {c->ux[c->cur], c->uy[c->cur], c->p};
        const int widths[3] = {c->itot + 1, c->itot + 2, c->itot + 2};
        bool first = true;
        for (int f = 0; f < 3; f++) {
          if (!hosts[f]) continue;
          rc = first ? rows_out(c, hosts[f], srcs[f], widths[f], rows, c->copy_stream, true)
                     : rows_out(c, hosts[f], srcs[f], widths[f], rows, c->stream);
          if (rc) return rc;
          first = false;
        }
        fields_queued = true;
      }
      if (s > 0 && (rc = finish(s - 1))) {
        if (cudaEventSynchronize(c->ev_step[s & 1]) == cudaSuccess) {
          c->step += 1;
          c->time += c->h_slots[s & 1].scal[0];
        }
        return rc;
      }
    }
    if (nsteps > 0) {
      const int rc = finish(nsteps - 1);
      if (rc) {
        cudaStreamSynchronize(c->copy_stream);
        return rc;
      }
      EIF_CK(c, cudaStreamSynchronize(c->stream));
    }
    if (fields_queued) EIF_CK(c, cudaStreamSynchronize(c->copy_stream));
  } else {
    for (int s = 0; s < nsteps; s++) {
      int rc = launch_decide_dt(c);
      if (rc) return rc;
      rc = eif_integrate(c, nullptr);
      if (rc) return rc;
      c->step += 1;
      c->time += c->dt_host;
    }
  }
  if (ft && !fields_queued) {
    const int rc = eif_pull_fluid(c, ft->ux, ft->uy, ft->p, nullptr);
    if (rc) return rc;
  }
  return ft ? check_records(c) : EIF_OK;
}

}  // namespace

int eif_advance(eif_ctx *c, int nsteps) { return advance(c, nsteps, nullptr); }

int eif_advance_pull(eif_ctx *c, int nsteps, double *ux, double *uy, double *p, int n, double *records) {
  if (!c || nsteps < 0 || (records && n != c->np)) return EIF_ERR_ARG;
  const FieldTargets ft{ux, uy, p};
  int rc = advance(c, nsteps, &ft);
  if (rc) return rc;
  if (records && (rc = eif_pull_particles(c, n, records))) return rc;
  return EIF_OK;
}

int eif_get_time(eif_ctx *c, int *step, double *time) {
  if (!c || !step || !time) return EIF_ERR_ARG;
  *step = c->step;
  *time = c->time;
  return EIF_OK;
}

int eif_set_time(eif_ctx *c, int step, double time) {
  if (!c) return EIF_ERR_ARG;
  c->step = step;
  c->time = time;
  return EIF_OK;
}

int eif_update_boundaries(eif_ctx *c) { return c ? launch_boundaries(c) : EIF_ERR_ARG; }
int eif_reset_particle_increments(eif_ctx *c) { return c ? launch_reset_increments(c) : EIF_ERR_ARG; }

int eif_compute_inertia(eif_ctx *c, int cn) {
  if (!c || (cn != 0 && cn != 1)) return c ? fail(c, EIF_ERR_ARG, "cnstep must be 0 or 1") : EIF_ERR_ARG;
  return launch_inertia(c, cn);
}

int eif_update_velocity(eif_ctx *c, int rk) {
  if (!c || !valid_rk(rk)) return c ? fail(c, EIF_ERR_ARG, "rkstep must be 0, 1 or 2") : EIF_ERR_ARG;
  return launch_predictor(c, rk);
}

int eif_exchange_momentum(eif_ctx *c) { return c ? launch_exchange(c) : EIF_ERR_ARG; }
int eif_update_momentum_field(eif_ctx *c) { return c ? launch_update_momentum_field(c) : EIF_ERR_ARG; }

int eif_compute_potential(eif_ctx *c, int rk) {
  if (!c || !valid_rk(rk)) return c ? fail(c, EIF_ERR_ARG, "rkstep must be 0, 1 or 2") : EIF_ERR_ARG;
  return launch_potential(c, rk, false);
}

int eif_correct_velocity(eif_ctx *c, int rk) {
  if (!c || !valid_rk(rk)) return c ? fail(c, EIF_ERR_ARG, "rkstep must be 0, 1 or 2") : EIF_ERR_ARG;
  return launch_correct(c, rk, false, false);
}

int eif_update_pressure(eif_ctx *c) { return c ? launch_update_pressure(c) : EIF_ERR_ARG; }

int eif_compute_collision_force(eif_ctx *c, int cn) {
  if (!c || (cn != 0 && cn != 1)) return c ? fail(c, EIF_ERR_ARG, "cnstep must be 0 or 1") : EIF_ERR_ARG;
  int rc = launch_collision(c, cn);
  if (rc) return rc;
  return sync_scalars(c);
}

int eif_increment_particles(eif_ctx *c, int rk, double *residual) {
  if (!c || !valid_rk(rk)) return c ? fail(c, EIF_ERR_ARG, "rkstep must be 0, 1 or 2") : EIF_ERR_ARG;
  int rc = launch_increment(c, rk);
  if (rc) return rc;
  if ((rc = sync_scalars(c))) return rc;
  if (residual) *residual = c->h_scal[1];
  return EIF_OK;
}

int eif_update_particles(eif_ctx *c) { return c ? launch_update_particles(c) : EIF_ERR_ARG; }

int eif_divergence(eif_ctx *c, double *divmax, double *divsum) {
  if (!c || !divmax || !divsum) return EIF_ERR_ARG;
  return launch_divergence(c, divmax, divsum);
}

int eif_momentum(eif_ctx *c, double *moms) {
  if (!c || !moms) return EIF_ERR_ARG;
  double q[4];
  int rc = launch_field_sums(c, q);
  if (rc) return rc;
  moms[0] = q[0];
  moms[1] = q[1];
  return EIF_OK;
}

int eif_energy(eif_ctx *c, double *energy) {
  if (!c || !energy) return EIF_ERR_ARG;
  double q[4];
  int rc = launch_field_sums(c, q);
  if (rc) return rc;
  energy[0] = q[2];
  energy[1] = q[3];
  return EIF_OK;
}

int eif_log_quantities(eif_ctx *c, double *q) {
  if (!c || !q) return EIF_ERR_ARG;
  int rc = launch_field_sums(c, q + 2);
  if (rc) return rc;
  return launch_divergence(c, q, q + 1);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// kernel timing
namespace eif {

static cudaEvent_t take_event(eif_ctx *c) {
  if (!c->prof.pool.empty()) {
    cudaEvent_t e = c->prof.pool.back();
    c->prof.pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

ProfScope::ProfScope(eif_ctx *c_, const char *name, int kernels) : c(c_), entry(-1), stop(nullptr) {
  if (!c->prof.enabled) return;
  auto &es = c->prof.entries;
  for (size_t k = 0; k < es.size(); k++) {
    if (es[k].name == name) { entry = (int)k; break; }
  }
  if (entry < 0) {
    es.push_back(Profiler::Entry{name, 0, 0.});
    entry = (int)es.size() - 1;
  }
  es[entry].launches += kernels;
  cudaEvent_t start = take_event(c);
  stop = take_event(c);
  cudaEventRecord(start, c->stream);
  c->prof.pending.push_back(Profiler::Pending{entry, start, stop});
}

ProfScope::~ProfScope() {
  if (entry >= 0) cudaEventRecord(stop, c->stream);
}

int profile_flush(eif_ctx *c) {
  if (c->prof.pending.empty()) return EIF_OK;
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  for (auto &p : c->prof.pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.start, p.stop) == cudaSuccess) c->prof.entries[p.entry].ms += ms;
    c->prof.pool.push_back(p.start);
    c->prof.pool.push_back(p.stop);
  }
  c->prof.pending.clear();
  return EIF_OK;
}

void profile_free(eif_ctx *c) {
  for (auto &p : c->prof.pending) { cudaEventDestroy(p.start); cudaEventDestroy(p.stop); }
  for (auto e : c->prof.pool) cudaEventDestroy(e);
  c->prof.pending.clear();
  c->prof.pool.clear();
}

}  // namespace eif

extern "C" {

int eif_profile_enable(eif_ctx *c, int enable) {
  if (!c) return EIF_ERR_ARG;
  int rc = profile_flush(c);
  c->prof.enabled = enable != 0;
  return rc;
}

int eif_profile_reset(eif_ctx *c) {
  if (!c) return EIF_ERR_ARG;
  int rc = profile_flush(c);
  c->prof.entries.clear();
  return rc;
}

int eif_profile_count(eif_ctx *c, int *count) {
  if (!c || !count) return EIF_ERR_ARG;
  int rc = profile_flush(c);
  *count = (int)c->prof.entries.size();
  return rc;
}

int eif_counters(eif_ctx *c, long long *counts) {
  if (!c || !counts) return EIF_ERR_ARG;
  unsigned long long v[3];
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  EIF_CK(c, cudaMemcpy(v, c->d_inc + 2, sizeof(v), cudaMemcpyDeviceToHost));
  for (int k = 0; k < 3; k++) counts[k] = (long long)v[k];
  return EIF_OK;
}

int eif_memo_count(eif_ctx *c, long long *tasks) {
  if (!c || !tasks) return EIF_ERR_ARG;
  unsigned long long v = 0;
  EIF_CK(c, cudaStreamSynchronize(c->stream));
  EIF_CK(c, cudaMemcpy(&v, c->d_inc + 5, sizeof(v), cudaMemcpyDeviceToHost));
  *tasks = (long long)v;
  return EIF_OK;
}

int eif_profile_get(eif_ctx *c, int k, char *name, int name_len, long long *launches, double *ms) {
  if (!c || k < 0 || k >= (int)c->prof.entries.size()) return EIF_ERR_ARG;
  int rc = profile_flush(c);
  const auto &e = c->prof.entries[k];
  if (name && name_len > 0) {
    strncpy(name, e.name.c_str(), (size_t)name_len - 1);
    name[name_len - 1] = 0;
  }
  if (launches) *launches = e.launches;
  if (ms) *ms = e.ms;
  return rc;
}

}  // extern "C"
