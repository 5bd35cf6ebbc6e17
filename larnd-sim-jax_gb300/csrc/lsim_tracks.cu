// Batch assembly of the tracks dataset on the device (TracksDataset,
// optimize/dataio.py:347-405): the batch's rows are gathered from a track
// table resident in HBM with their event ids replaced by the batch-local
// ids (remap_event_ids_to_local, :47-61), and a batch is padded to a fixed
// row count with invalidated rows (pad_batch / _invalidate_rows, :347-373).
//
// k_gather_rows: one warp per output row, lanes over the columns (rows are
// at most 96 floats), so every row is one or three coalesced loads and
// stores.  A row index outside the table sets the status word and writes
// nothing.  k_pad_rows: one warp per row it may rewrite.
#include "lsim_internal.cuh"

namespace lsim {
namespace {

constexpr int kGatherWarps = 8;
constexpr int kMaxTrackFields = 96;

__global__ void __launch_bounds__(kGatherWarps * kWarp) k_gather_rows(const float *__restrict__ table, int64_t n_table,
                                                                     int32_t n_fields,
                                                                     const int64_t *__restrict__ rows, int64_t n_rows,
                                                                     int32_t event_col,
                                                                     const float *__restrict__ event_values,
                                                                     float *__restrict__ out,
                                                                     int32_t *__restrict__ status) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (int64_t)blockIdx.x * kGatherWarps + (threadIdx.x >> 5);
  if (r >= n_rows) return;
  const int64_t src = rows[r];
  if (src < 0 || src >= n_table) {
    if (lane == 0) atomicCAS(status, 0, LSIM_ERR_INVALID);
    return;
  }
  const float *in = table + src * n_fields;
  float *o = out + r * n_fields;
  for (int c = lane; c < n_fields; c += kWarp) o[c] = (c == event_col && event_values) ? event_values[r] : in[c];
}

struct PadRoles {
  int8_t role[kMaxTrackFields];  // 0: kept (0 in padding rows), 1: zeroed, 2: set to -1, 3: the event column
};

// Rows [0, n_rows) whose event id is >= 0 but whose integer part is not a
// local event id are invalidated (only when n_local_events >= 0); rows
// [n_rows, target_rows) become padding.  One warp per row: lane 0's read
// of the event id reaches the other lanes by shuffle before any lane writes.
__global__ void __launch_bounds__(kGatherWarps * kWarp) k_pad_rows(float *__restrict__ batch, int64_t n_rows,
                                                                  int64_t first_row, int64_t target_rows,
                                                                  int32_t n_fields, int32_t event_col, PadRoles roles,
                                                                  int64_t n_local_events) {
  const int lane = threadIdx.x & 31;
  const int64_t r = first_row + (int64_t)blockIdx.x * kGatherWarps + (threadIdx.x >> 5);
  if (r >= target_rows) return;
  float *row = batch + r * n_fields;
  bool invalid = r >= n_rows;
  if (!invalid) {
    const float ev = __shfl_sync(0xffffffffu, lane == 0 ? row[event_col] : 0.f, 0);
    if (ev >= 0.f) {
      const long long li = (long long)ev;  // numpy's astype(int64): truncation
      invalid = li < 0 || li >= n_local_events;
    }
  }
  if (!invalid) return;
  for (int c = lane; c < n_fields; c += kWarp) {
    const int role = roles.role[c];
    if (role == 3 || role == 2) {
      row[c] = -1.f;
    } else if (role == 1 || r >= n_rows) {
      row[c] = 0.f;
    }
  }
}

}  // namespace

int run_gather_tracks(const float *table, int64_t n_table, int32_t n_fields, const int64_t *rows, int64_t n_rows,
                      int32_t event_col, const float *event_values, float *out, int32_t *status, cudaStream_t st) {
  if (n_rows == 0) return LSIM_OK;
  const int64_t blocks = (n_rows + kGatherWarps - 1) / kGatherWarps;
  k_gather_rows<<<(unsigned)blocks, kGatherWarps * kWarp, 0, st>>>(table, n_table, n_fields, rows, n_rows, event_col,
                                                                  event_values, out, status);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

int run_pad_tracks(float *batch, int64_t n_rows, int64_t target_rows, int32_t n_fields, int32_t event_col,
                   const int8_t *col_roles, int64_t n_local_events, cudaStream_t st) {
  PadRoles roles{};
  for (int c = 0; c < n_fields; ++c) roles.role[c] = col_roles ? col_roles[c] : 0;
  roles.role[event_col] = 3;
  const int64_t first = n_local_events >= 0 ? 0 : n_rows;
  const int64_t count = target_rows - first;
  if (count <= 0) return LSIM_OK;
  const int64_t blocks = (count + kGatherWarps - 1) / kGatherWarps;
  k_pad_rows<<<(unsigned)blocks, kGatherWarps * kWarp, 0, st>>>(batch, n_rows, first, target_rows, n_fields, event_col,
                                                                roles, n_local_events);
  return cudaGetLastError() == cudaSuccess ? LSIM_OK : LSIM_ERR_CUDA;
}

}  // namespace lsim
