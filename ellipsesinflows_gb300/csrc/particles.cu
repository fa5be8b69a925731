// Particle kernels: soft-sphere collisions between ellipses (via equivalent
// circles), Crank-Nicolson increments, and the final velocity/position update.
//
// Reference functions restated here (NaokiHori/EllipsesInFlows):
//   compute_evolute, find_equivalent_circle(s)   src/suspensions/collision.c:75-154
//   compute_collision_force_p_p / _p_w           src/suspensions/collision.c:156-304
//   suspensions_compute_collision_force          src/suspensions/collision.c:306-367
//   compute_curvature                            src/ellipse.c:17-28
//   suspensions_reset_particle_increments        src/suspensions/reset.c:7-18
//   suspensions_increment_particles              src/suspensions/increment.c:10-72
//   suspensions_update_particles                 src/suspensions/update.c:8-34,61-65
//
// Collision force on particle k accumulates, as in the reference, over the
// pairs in the order of the pair matrix (partners m = 0..N-1, m != k) and
// then the walls at x = 0 and x = lx. Candidate pairs are found by a tiled scan
// (a conservative single-precision distance test, then the exact double-precision
// bounding-circle test of collision.c:173-189); one warp per particle then
// evaluates its candidates one per lane and sums them in partner order.
#include "particle_device.cuh"
#include <algorithm>

namespace {

__global__ void __launch_bounds__(PAIR_WARPS * 32) k_collision(double *__restrict__ P, int pcap, int np, int cn,
                                                               double ly, double lx, unsigned *__restrict__ flags) {
  collision_block(P, pcap, np, cn, ly, lx, flags, blockIdx.x);
}

__global__ void k_reset(double *__restrict__ P, int pcap, int np) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n < np) reset_particle(P, pcap, n);
}

// increment.c:10-72; residual = max |change of the increments|, combined over
// blocks as an integer max of the IEEE bits of non-negative doubles (independent
// of the order). The FP64 work is spread over many SMs: one SM alone has only a
// few FP64 lanes.
__global__ void k_increment(double *__restrict__ P, int pcap, int np, double gamma, double Fr2,
                            double *__restrict__ scal, unsigned long long *__restrict__ res_bits,
                            unsigned *__restrict__ counter, unsigned *__restrict__ arrivals,
                            unsigned long long *__restrict__ total, cudaGraphConditionalHandle handle,
                            int use_handle) {
  const double dt = scal[0];
  double res = 0.;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < np; n += gridDim.x * blockDim.x)
    res = increment_particle(P, pcap, n, gamma, Fr2, dt, res);
  res = eifd::warp_max(res);
  __shared__ double s[32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = res;
  __syncthreads();
  __shared__ bool last;
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) res = fmax(res, s[w]);
    if (res > 0.) atomicMax(res_bits, (unsigned long long)__double_as_longlong(res));
    // the last block to finish publishes the residual (its maximum is complete)
    __threadfence();
    last = atomicAdd(arrivals, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    *arrivals = 0u;
    const double r = __longlong_as_double((long long)atomicExch(res_bits, 0ull));
    scal[1] = r;
    *total += 1ull;   // sub-iterations run (eif_counters)
    // inside a step graph: the condition of the sub-iteration loop (main.c:40-48):
    // continue while the residual is not below 1e-8 and at most 101 sub-iterations ran
    if (use_handle) {
      const unsigned count = ++*counter;
      cudaGraphSetConditional(handle, (!(r < 1.e-8) && count <= 101u) ? 1u : 0u);
    }
  }
}


// update.c:8-34
__global__ void k_update(double *__restrict__ P, int pcap, int np, double ly) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n < np) update_particle(P, pcap, n, ly);
}

}  // namespace

namespace eif {

int launch_collision(eif_ctx *c, int cn) {
  if (c->np == 0) return EIF_OK;
  EIF_PROF(c, "collision", 1);
  k_collision<<<(c->np + PAIR_WARPS - 1) / PAIR_WARPS, PAIR_WARPS * 32, 0, c->stream>>>(c->P, c->pcap, c->np, cn,
                                                                                      c->ly, c->lx, c->d_flags);
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}

int launch_reset_increments(eif_ctx *c) {
  c->incr_zero = true;
  // in a batch graph the stage kernel before this front has reset the increments
  if (c->np == 0 || c->reset_in_stage_kernel) return EIF_OK;
  EIF_PROF(c, "particle_reset", 1);
  k_reset<<<(c->np + 127) / 128, 128, 0, c->stream>>>(c->P, c->pcap, c->np);
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}

int launch_increment(eif_ctx *c, int rk) {
  c->incr_zero = false;
  const double Fr = c->cfg.Fr;
  EIF_PROF(c, "particle_increment", 1);
  // FP64-heavy per particle: small blocks spread the particles over many SMs
  const int blocks = std::max(1, std::min((c->np + 31) / 32, c->sms * 4));
  unsigned *counter = reinterpret_cast<unsigned *>(c->d_inc + 1);   // low word: loop counter
  k_increment<<<blocks, 32, 0, c->stream>>>(c->P, c->pcap, c->np, rk_coef(rk).gamma, Fr * Fr, c->d_scal, c->d_inc,
                                             counter, counter + 1, c->d_inc + 2, c->loop_handle,
                                             c->in_loop ? 1 : 0);
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}

int launch_update_particles(eif_ctx *c) {
  c->boxes_x_valid = false;
  c->weights_x_valid = false;
  if (c->np == 0) return EIF_OK;
  EIF_PROF(c, "particle_update", 1);
  k_update<<<(c->np + 127) / 128, 128, 0, c->stream>>>(c->P, c->pcap, c->np, c->ly);
  EIF_LAUNCH_CK(c);
  return EIF_OK;
}

}  // namespace eif
