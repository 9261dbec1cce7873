// Batches of independent FFT grids (the multiple-grids use of
// src/fft_common.f90:381-479, where an application drives several engines in
// turn) with one CUDA graph holding the forward and backward transforms of
// every grid, replayed with a single launch call.
#include <string>
#include <vector>

#include "gbfft.h"
#include "gbfft_internal.h"

namespace {

constexpr unsigned kBatchMagic = 0x47424254u;  // "GBBT"

struct Item {
  gbfft_engine_t eng;
  const void* real;
  void* spec;
};

}  // namespace

struct gbfft_batch_s {
  unsigned magic = kBatchMagic;
  std::vector<Item> items;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

bool valid(gbfft_batch_t b) { return b && b->magic == kBatchMagic; }

void drop_graph(gbfft_batch_t b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

int run_forward(gbfft_batch_t b, cudaStream_t st) {
  for (const Item& it : b->items) {
    int rc = gbfft_exec_r2c(it.eng, it.real, it.spec, st);
    if (rc) return rc;
  }
  return GBFFT_OK;
}

int run_backward(gbfft_batch_t b, cudaStream_t st) {
  for (const Item& it : b->items) {
    int rc = gbfft_exec_c2r(it.eng, it.spec, const_cast<void*>(it.real), st);
    if (rc) return rc;
  }
  return GBFFT_OK;
}

}  // namespace

extern "C" {

int gbfft_batch_create(gbfft_batch_t* batch) {
  if (!batch) return gbfft::set_error(GBFFT_ERR_INVALID, "null output pointer");
  *batch = new (std::nothrow) gbfft_batch_s();
  if (!*batch) return gbfft::set_error(GBFFT_ERR_ALLOC, "host allocation failed");
  return GBFFT_OK;
}

int gbfft_batch_add(gbfft_batch_t b, gbfft_engine_t eng, const void* d_real, void* d_spec) {
  if (!valid(b)) return gbfft::set_error(GBFFT_ERR_INVALID, "not a batch");
  if (!eng || !d_real || !d_spec) return gbfft::set_error(GBFFT_ERR_INVALID, "null argument");
  int ph[3], sp[3];
  int rc = gbfft_engine_get_sizes(eng, ph, sp);
  if (rc) return rc;
  drop_graph(b);
  b->items.push_back({eng, d_real, d_spec});
  return GBFFT_OK;
}

int gbfft_batch_forward(gbfft_batch_t b, void* stream) {
  if (!valid(b)) return gbfft::set_error(GBFFT_ERR_INVALID, "not a batch");
  return run_forward(b, (cudaStream_t)stream);
}

int gbfft_batch_backward(gbfft_batch_t b, void* stream) {
  if (!valid(b)) return gbfft::set_error(GBFFT_ERR_INVALID, "not a batch");
  return run_backward(b, (cudaStream_t)stream);
}

int gbfft_batch_graph_build(gbfft_batch_t b, void* stream) {
  if (!valid(b)) return gbfft::set_error(GBFFT_ERR_INVALID, "not a batch");
  if (!stream) return gbfft::set_error(GBFFT_ERR_INVALID, "graph capture needs a non-default stream");
  drop_graph(b);
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess)
    return gbfft::set_error(GBFFT_ERR_CUDA, (std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e)).c_str());
  int rc = run_forward(b, st);
  if (!rc) rc = run_backward(b, st);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(st, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess)
    return gbfft::set_error(GBFFT_ERR_CUDA, (std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e)).c_str());
  e = cudaGraphInstantiate(&b->exec, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    b->exec = nullptr;
    return gbfft::set_error(GBFFT_ERR_CUDA, (std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e)).c_str());
  }
  b->graph = g;
  return GBFFT_OK;
}

int gbfft_batch_graph_launch(gbfft_batch_t b, void* stream) {
  if (!valid(b)) return gbfft::set_error(GBFFT_ERR_INVALID, "not a batch");
  if (!b->exec) return gbfft::set_error(GBFFT_ERR_STATE, "graph not built");
  cudaError_t e = cudaGraphLaunch(b->exec, (cudaStream_t)stream);
  if (e != cudaSuccess)
    return gbfft::set_error(GBFFT_ERR_CUDA, (std::string("cudaGraphLaunch: ") + cudaGetErrorString(e)).c_str());
  return GBFFT_OK;
}

int gbfft_batch_destroy(gbfft_batch_t b) {
  if (!b) return GBFFT_OK;
  if (!valid(b)) return gbfft::set_error(GBFFT_ERR_INVALID, "not a batch");
  drop_graph(b);
  b->magic = 0;
  delete b;
  return GBFFT_OK;
}

}  // extern "C"
