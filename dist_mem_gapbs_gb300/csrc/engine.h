// Internal host-side definitions shared by the translation units of libgbbfs:
// the graph handle, error reporting and the CUDA-call helpers.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "bfs_common.cuh"
#include "gbbfs.h"

namespace gbbfs {

// Detail of the last failure on the calling thread (gbbfs_last_error).
inline std::string& last_error() {
  thread_local std::string msg;
  return msg;
}

struct MsState;   // multi-source BFS buffers of a handle (msbfs.cu)
void msbfs_release(MsState* ms);
struct BcState;   // BC BFS-phase buffers of a handle (bc.cu)
void bc_release(BcState* b);

}  // namespace gbbfs

struct gbbfs_graph;

namespace gbbfs {

// Asynchronous batch primitives of the multi-source search (msbfs.cu), used
// by the query server.  Two depth buffers per handle; batches on one handle
// run in stream order, batches on different handles overlap on the device.
size_t ms_state_bytes(int64_t n, int64_t m, int64_t W, int depth_bytes);  // HBM a handle's state takes
int ms_prepare(gbbfs_graph* g, int depth_bytes);   // allocate (or keep) the state
int ms_lanes(const gbbfs_graph* g);
// SMs a batch's cooperative grid spans on this handle (0: all of them); the
// handle's captured batch graphs are remade at their next launch.
int ms_set_grid_sms(gbbfs_graph* g, int sms);
int ms_launch(gbbfs_graph* g, int buf, const int32_t* sources, int k);
bool ms_ready(gbbfs_graph* g, int buf);            // batch in `buf` has finished
int ms_finish(gbbfs_graph* g, int buf);            // wait, then report its status
void* ms_depth(gbbfs_graph* g, int buf);           // device rows of `buf`
cudaEvent_t ms_done_event(gbbfs_graph* g, int buf);
void ms_mark_copied(gbbfs_graph* g, int buf, cudaStream_t s);  // copies out of `buf` queued on s
// Device time (ms) of the search kernel of the finished batch in `buf`, from
// its own start and end stamps (a cooperative kernel runs alone once started,
// so this excludes waits for other work).
double ms_kernel_ms(const gbbfs_graph* g, int buf);
// Device clock (%globaltimer, ns) at that kernel's start and end.
void ms_kernel_stamps(const gbbfs_graph* g, int buf, uint64_t* begin_ns, uint64_t* end_ns);
// Indices of sources[0..k) in the order to batch them (gbbfs_msbfs_order).
int ms_order(gbbfs_graph* g, const int32_t* sources, int64_t k, int32_t* order);

// Stable LSD radix sort of len 64-bit keys on their low key_bits bits
// (gpu_build.cu); keys and tmp hold len each, *out is the sorted one.
int radix_sort64(uint64_t* keys, uint64_t* tmp, int64_t len, int key_bits, cudaStream_t s,
                 uint64_t** out);

// Single-source searches queued without waiting (bfs_engine.cu), for the
// query server.  bfs_enqueue queues one search from `source` on the handle's
// stream: its parameters come from the caller's pinned block of
// kSearchParamBytes, which must stay untouched until the search has run;
// depths are kept in bfs_depth(g) and parents in the handle's own array, and
// bfs_error_word(g) (device) holds the search's error status.  The caller
// orders its reads of them on the same stream, before the next search.
constexpr size_t kSearchParamBytes = offsetof(DevState, edges_to_check);
int bfs_enqueue(gbbfs_graph* g, int32_t source, void* h_params);
const int32_t* bfs_depth(const gbbfs_graph* g);
// Replace the handle's stream by one of the given priority (lower numbers
// run first, cudaDeviceGetStreamPriorityRange); waits for the old stream.
int graph_set_stream_priority(gbbfs_graph* g, int priority);
const int32_t* bfs_error_word(const gbbfs_graph* g);

// A handle from a CSR in device memory (bfs_engine.cu): offsets int64[n+1]
// and neighbours int32[m], copied into the handle.
int graph_create_device(const int64_t* d_off, const int32_t* d_nbr, int64_t n, int64_t m,
                        gbbfs_graph** out);

}  // namespace gbbfs

#define GB_CUDA(call)                                                              \
  do {                                                                             \
    cudaError_t err_ = (call);                                                     \
    if (err_ != cudaSuccess) {                                                     \
      ::gbbfs::last_error() = std::string(#call) + ": " + cudaGetErrorString(err_); \
      return GBBFS_ERR_CUDA;                                                       \
    }                                                                              \
  } while (0)

#define GB_TRY(x)            \
  do {                       \
    int st_ = (x);           \
    if (st_ != GBBFS_OK) {   \
      return st_;            \
    }                        \
  } while (0)

struct gbbfs_graph {
  int64_t n = 0, m = 0, W = 0;
  bool off32 = true;
  int shift = 32;           // packed queue counter: (count << shift) | edges
  int device = 0;
  int sms = 0;
  void* off = nullptr;      // uint32_t* or unsigned long long*
  int32_t* nbr = nullptr;
  int2* head = nullptr;     // first two neighbours of every vertex (-1 past its degree)
  uint32_t* iso = nullptr;
  uint32_t* visited = nullptr;
  uint32_t* bm[2] = {nullptr, nullptr};
  int32_t* parent = nullptr;
  int32_t* last_parent = nullptr;   // parent array of the last search
  int32_t* depth = nullptr;
  int32_t* qv[2] = {nullptr, nullptr};
  void* qs[2] = {nullptr, nullptr};
  gbbfs::DevCounters* ctr = nullptr;
  gbbfs::DevState* st = nullptr;
  gbbfs::DevState* h_st = nullptr;  // pinned mirror (params in, header + trace out)
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
  std::vector<cudaEvent_t> step_ev;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int grid_init = 0, grid_td = 0, grid_bu = 0, grid_q2b = 0, grid_b2q = 0, grid_tdb = 0,
      grid_sweep = 0;
  int64_t device_bytes = 0;
  bool have_result = false;
  bool result_depth = false;
  gbbfs::MsState* ms = nullptr;
  gbbfs::BcState* bc = nullptr;
  // Batching key per vertex (host): BFS depth from the highest-degree vertex
  // (255 = unreached) << 8 | (255 - min(degree, 255)).  Made on first use.
  std::vector<uint16_t> batch_key;
  // gbbfs_bfs_many: the two parent arrays its searches alternate between,
  // and the stream that copies them out.
  int32_t* stage[2] = {nullptr, nullptr};
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t staged[2] = {nullptr, nullptr};
  cudaEvent_t copied[2] = {nullptr, nullptr};
  // Its searches without stats: parameters and read-back headers per slot
  // (pinned), so a search is queued before the one before it has finished.
  gbbfs::DevState* h_slot = nullptr;
};
