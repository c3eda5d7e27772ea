// Sample gates for the proposal-gated render: which coarse samples, and which
// members of the sorted coarse+fine union, the NeRF MLP evaluates.
//
// The learned proposal's per-bin weights say where a ray can carry density.
// Coarse samples whose proposal weight is at most `tau` are not evaluated
// (their sigma is 0); the same coarse samples are skipped again when they
// reappear in the fine pass's sorted union, while every fine draw is
// evaluated. The gates compact the kept samples into a row map that the MLP
// kernels read directly (RowMap), with the count left on the device.
//
// One warp per ray: a ballot per 32 samples, one atomicAdd per ray for its
// segment of the row map (rays land in any order, a ray's samples in order;
// each MLP row is computed independently, so the order does not change any
// result).
#include "common.cuh"
#include "mlp_internal.cuh"

namespace nerfgb {

__global__ void gate_coarse_kernel(const float *__restrict__ w, int R, int S, float tau,
                                   unsigned char *__restrict__ mask, int *__restrict__ row_map,
                                   int *__restrict__ count) {
  const int ray = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (ray >= R) return;  // whole warps
  const long long row0 = (long long)ray * S;
  int total = 0;
  for (int j0 = 0; j0 < S; j0 += 32) {
    const int j = j0 + lane;
    const bool on = j < S && w[row0 + j] > tau;  // NaN: off
    total += __popc(__ballot_sync(0xffffffffu, on));
  }
  int base = 0;
  if (lane == 0 && total > 0) base = atomicAdd(count, total);
  base = __shfl_sync(0xffffffffu, base, 0);
  for (int j0 = 0; j0 < S; j0 += 32) {
    const int j = j0 + lane;
    const bool on = j < S && w[row0 + j] > tau;
    const unsigned b = __ballot_sync(0xffffffffu, on);
    if (j < S) mask[row0 + j] = on ? 1 : 0;
    if (on) row_map[NG_IDX(base + __popc(b & ((1u << lane) - 1u)), (long long)R * S, kSiteGateCoarse)] = (int)(row0 + j);
    base += __popc(b);
  }
}

__global__ void gate_fine_kernel(const int *__restrict__ perm, const unsigned char *__restrict__ mask_c,
                                 const int *__restrict__ piece, int R, int Sc, int S, int *__restrict__ row_map,
                                 int *__restrict__ count) {
  const int ray = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (ray >= R) return;
  const long long row0 = (long long)ray * S;
  auto keep = [&](int j) -> bool {
    if (j >= S) return false;
    const int p = (int)NG_IDX(perm[row0 + j], S, kSiteGateFinePerm);
    // a coarse sample whose gate is on, or a fine draw (given the draws'
    // bins: one whose coarse bin's gate is on)
    if (p >= Sc) {
      if (!piece) return true;
      const int bin = (int)NG_IDX(piece[(long long)ray * (S - Sc) + (p - Sc)], Sc, kSiteGateFinePiece);
      return mask_c[(long long)ray * Sc + bin] != 0;
    }
    return p >= 0 && mask_c[(long long)ray * Sc + p] != 0;
  };
  int total = 0;
  for (int j0 = 0; j0 < S; j0 += 32) total += __popc(__ballot_sync(0xffffffffu, keep(j0 + lane)));
  int base = 0;
  if (lane == 0 && total > 0) base = atomicAdd(count, total);
  base = __shfl_sync(0xffffffffu, base, 0);
  for (int j0 = 0; j0 < S; j0 += 32) {
    const int j = j0 + lane;
    const bool on = keep(j);
    const unsigned b = __ballot_sync(0xffffffffu, on);
    if (on) row_map[NG_IDX(base + __popc(b & ((1u << lane) - 1u)), (long long)R * S, kSiteGateFine)] = (int)(row0 + j);
    base += __popc(b);
  }
}

static int gate_grid(int R) { return (int)(((long long)R * 32 + 255) / 256); }

int launch_gate_coarse(const float *w, int R, int S, float tau, unsigned char *mask, int *row_map, int *count,
                       cudaStream_t stream) {
  if (R == 0) return NERFGB_OK;
  gate_coarse_kernel<<<gate_grid(R), 256, 0, stream>>>(w, R, S, tau, mask, row_map, count);
  return launch_status();
}

int launch_gate_fine(const int *perm, const unsigned char *mask_c, const int *piece, int R, int Sc, int S,
                     int *row_map, int *count, cudaStream_t stream) {
  if (R == 0) return NERFGB_OK;
  gate_fine_kernel<<<gate_grid(R), 256, 0, stream>>>(perm, mask_c, piece, R, Sc, S, row_map, count);
  return launch_status();
}

}  // namespace nerfgb

using namespace nerfgb;

extern "C" int nerfgb_gate_coarse(const float *weights, int n_rays, int n_samples, float tau, unsigned char *mask,
                                  int *row_map, int *count, void *stream) {
  if (n_rays < 0 || n_samples < 1 || (long long)n_rays * n_samples > 0x7fffffffLL) return NERFGB_E_INVALID_ARG;
  if (n_rays == 0) return NERFGB_OK;
  if (!weights || !mask || !row_map || !count) return NERFGB_E_INVALID_ARG;
  return launch_gate_coarse(weights, n_rays, n_samples, tau, mask, row_map, count, as_stream(stream));
}

extern "C" int nerfgb_gate_fine(const int *sort_perm, const unsigned char *mask_coarse, const int *piece_idxs,
                                int n_rays, int n_coarse, int n_samples, int *row_map, int *count, void *stream) {
  if (n_rays < 0 || n_coarse < 1 || n_samples < n_coarse || (long long)n_rays * n_samples > 0x7fffffffLL)
    return NERFGB_E_INVALID_ARG;
  if (n_rays == 0) return NERFGB_OK;
  if (!sort_perm || !mask_coarse || !row_map || !count) return NERFGB_E_INVALID_ARG;
  return launch_gate_fine(sort_perm, mask_coarse, piece_idxs, n_rays, n_coarse, n_samples, row_map, count,
                          as_stream(stream));
}

#ifdef NERF_BOUNDS_CHECK
namespace nerfgb {
NG_BOUNDS_READER(bounds_read_gate)
}  // namespace nerfgb
#endif
