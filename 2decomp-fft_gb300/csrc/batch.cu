// Batches of independent FFT grids (the multiple-grids use of
// src/fft_common.f90:381-479, where an application drives several engines in
// turn).  Two ways to run a batch:
//   per-grid loop   every grid's passes as their own launches, grid after
//                   grid (what the reference does);
//   persistent      every pass of every grid in one launch (batch_kernel.cu),
//                   for FP32 grids whose line lengths the batch kernel runs.
// Either can be captured, forward then backward, into one CUDA graph.
#include <string>
#include <vector>

#include "gbfft.h"
#include "gbfft_internal.h"

using namespace gbfft;

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
  bool persistent = true;  // use the one-launch path when the batch allows it
  // device descriptors of the persistent path, built on first use per mask
  int built_mask = 0;
  bool eligible = false;
  BatchDesc* d_desc = nullptr;
  long long* d_prefix = nullptr;
  int* d_sync = nullptr;
  int ndesc = 0;
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

void drop_desc(gbfft_batch_t b) {
  if (b->d_desc) dev_free(b->d_desc);
  if (b->d_prefix) dev_free(b->d_prefix);
  if (b->d_sync) dev_free(b->d_sync);
  b->d_desc = nullptr;
  b->d_prefix = nullptr;
  b->d_sync = nullptr;
  b->ndesc = 0;
  b->built_mask = 0;
  b->eligible = false;
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

// Descriptors of every pass of every item (forward if mask & 1, then
// backward if mask & 2), stage-major, each depending on the previous pass of
// its own item.  Sets b->eligible = false when some pass cannot run in the
// batch kernel (then nothing is allocated).
int build_desc(gbfft_batch_t b, int mask) {
  drop_desc(b);
  std::vector<std::vector<PassInfo>> per(b->items.size());
  for (size_t g = 0; g < b->items.size(); ++g) {
    const Item& it = b->items[g];
    if (engine_precision(it.eng) != GBFFT_PREC_SINGLE) {
      b->built_mask = mask;
      return GBFFT_OK;
    }
    PassInfo buf[8];
    int n = 0;
    if (mask & 1) {
      int rc = engine_passes(it.eng, 0, it.real, it.spec, buf, 8, &n);
      if (rc) return rc;
      per[g].insert(per[g].end(), buf, buf + n);
    }
    if (mask & 2) {
      int rc = engine_passes(it.eng, 1, it.spec, const_cast<void*>(it.real), buf, 8, &n);
      if (rc) return rc;
      per[g].insert(per[g].end(), buf, buf + n);
    }
    for (const PassInfo& p : per[g])
      if ((p.a.fast != 1 && p.a.fast != 2) || !batch_length(p.a.n)) {
        b->built_mask = mask;
        return GBFFT_OK;
      }
  }
  size_t stages = 0;
  for (auto& v : per) stages = v.size() > stages ? v.size() : stages;
  std::vector<BatchDesc> desc;
  std::vector<long long> prefix(1, 0);
  std::vector<int> last(per.size(), -1);
  for (size_t s = 0; s < stages; ++s)
    for (size_t g = 0; g < per.size(); ++g) {
      if (s >= per[g].size()) continue;
      const PassInfo& p = per[g][s];
      BatchDesc d;
      d.a = p.a;
      const int le = batch_tile_lines(p.a.n, p.contiguous);
      d.a.L = le + 1;
      d.code = 2 * p.kind + (p.contiguous ? 0 : 1);
      d.dep = last[g];
      d.nu = p.a.nlines;
      d.lines = p.contiguous ? (long long)p.a.nlines : (long long)p.a.nlines * p.a.nv;
      last[g] = (int)desc.size();
      desc.push_back(d);
      prefix.push_back(prefix.back() + (d.lines + le - 1) / le);
    }
  b->ndesc = (int)desc.size();
  cudaError_t e = dev_malloc((void**)&b->d_desc, desc.size() * sizeof(BatchDesc));
  if (e == cudaSuccess) e = dev_malloc((void**)&b->d_prefix, prefix.size() * sizeof(long long));
  if (e == cudaSuccess) e = dev_malloc((void**)&b->d_sync, (desc.size() + 2) * sizeof(int));
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_desc, desc.data(), desc.size() * sizeof(BatchDesc), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_prefix, prefix.data(), prefix.size() * sizeof(long long), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    drop_desc(b);
    return set_error(GBFFT_ERR_ALLOC, (std::string("batch descriptors: ") + cudaGetErrorString(e)).c_str());
  }
  b->built_mask = mask;
  b->eligible = true;
  return GBFFT_OK;
}

int run(gbfft_batch_t b, int mask, cudaStream_t st) {
  if (b->items.empty()) return GBFFT_OK;
  if (b->persistent) {
    if (b->built_mask != mask) {
      int rc = build_desc(b, mask);
      if (rc) return rc;
    }
    if (b->eligible) {
      cudaError_t e = launch_batch_f32(b->d_desc, b->d_prefix, b->ndesc, b->d_sync, b->ndesc + 2, st);
      if (e != cudaSuccess)
        return set_error(GBFFT_ERR_CUDA, (std::string("batch launch: ") + cudaGetErrorString(e)).c_str());
      return GBFFT_OK;
    }
  }
  int rc = GBFFT_OK;
  if (mask & 1) rc = run_forward(b, st);
  if (!rc && (mask & 2)) rc = run_backward(b, st);
  return rc;
}

}  // namespace

extern "C" {

int gbfft_batch_create(gbfft_batch_t* batch) {
  if (!batch) return set_error(GBFFT_ERR_INVALID, "null output pointer");
  *batch = new (std::nothrow) gbfft_batch_s();
  if (!*batch) return set_error(GBFFT_ERR_ALLOC, "host allocation failed");
  return GBFFT_OK;
}

int gbfft_batch_add(gbfft_batch_t b, gbfft_engine_t eng, const void* d_real, void* d_spec) {
  if (!valid(b)) return set_error(GBFFT_ERR_INVALID, "not a batch");
  if (!eng || !d_real || !d_spec) return set_error(GBFFT_ERR_INVALID, "null argument");
  int ph[3], sp[3];
  int rc = gbfft_engine_get_sizes(eng, ph, sp);
  if (rc) return rc;
  drop_graph(b);
  drop_desc(b);
  b->items.push_back({eng, d_real, d_spec});
  return GBFFT_OK;
}

int gbfft_batch_set_persistent(gbfft_batch_t b, int enable) {
  if (!valid(b)) return set_error(GBFFT_ERR_INVALID, "not a batch");
  b->persistent = enable != 0;
  drop_graph(b);
  return GBFFT_OK;
}

int gbfft_batch_run(gbfft_batch_t b, int mask, void* stream) {
  if (!valid(b)) return set_error(GBFFT_ERR_INVALID, "not a batch");
  if (mask < 1 || mask > 3) return set_error(GBFFT_ERR_INVALID, "mask must be 1, 2 or 3");
  return run(b, mask, (cudaStream_t)stream);
}

int gbfft_batch_info(gbfft_batch_t b, int* persistent, int* launches_per_run) {
  if (!valid(b)) return set_error(GBFFT_ERR_INVALID, "not a batch");
  if (b->persistent && b->built_mask != 3) {
    int rc = build_desc(b, 3);
    if (rc) return rc;
  }
  const bool p = b->persistent && b->eligible;
  if (persistent) *persistent = p ? 1 : 0;
  if (launches_per_run) *launches_per_run = p ? 1 : -1;
  return GBFFT_OK;
}

int gbfft_batch_status(gbfft_batch_t b) {
  if (!valid(b)) return set_error(GBFFT_ERR_INVALID, "not a batch");
  if (!b->d_sync) return GBFFT_OK;
  int flag = 0;
  cudaError_t e = cudaMemcpy(&flag, b->d_sync + 1, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return set_error(GBFFT_ERR_CUDA, cudaGetErrorString(e));
  if (flag == 1) return set_error(GBFFT_ERR_TIMEOUT, "a batch tile gave up waiting for its previous pass");
  if (flag) return set_error(GBFFT_ERR_UNSUPPORTED, "a batch tile had a line length the kernel does not run");
  return GBFFT_OK;
}

int gbfft_batch_forward(gbfft_batch_t b, void* stream) {
  if (!valid(b)) return set_error(GBFFT_ERR_INVALID, "not a batch");
  return run_forward(b, (cudaStream_t)stream);
}

int gbfft_batch_backward(gbfft_batch_t b, void* stream) {
  if (!valid(b)) return set_error(GBFFT_ERR_INVALID, "not a batch");
  return run_backward(b, (cudaStream_t)stream);
}

int gbfft_batch_graph_build(gbfft_batch_t b, void* stream) {
  if (!valid(b)) return set_error(GBFFT_ERR_INVALID, "not a batch");
  if (!stream) return set_error(GBFFT_ERR_INVALID, "graph capture needs a non-default stream");
  drop_graph(b);
  // descriptors are uploaded before capture (no synchronous copies inside)
  if (b->persistent && b->built_mask != 3) {
    int rc = build_desc(b, 3);
    if (rc) return rc;
  }
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess)
    return set_error(GBFFT_ERR_CUDA, (std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e)).c_str());
  int rc = run(b, 3, st);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(st, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess)
    return set_error(GBFFT_ERR_CUDA, (std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e)).c_str());
  e = cudaGraphInstantiate(&b->exec, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    b->exec = nullptr;
    return set_error(GBFFT_ERR_CUDA, (std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e)).c_str());
  }
  b->graph = g;
  return GBFFT_OK;
}

int gbfft_batch_graph_launch(gbfft_batch_t b, void* stream) {
  if (!valid(b)) return set_error(GBFFT_ERR_INVALID, "not a batch");
  if (!b->exec) return set_error(GBFFT_ERR_STATE, "graph not built");
  cudaError_t e = cudaGraphLaunch(b->exec, (cudaStream_t)stream);
  if (e != cudaSuccess)
    return set_error(GBFFT_ERR_CUDA, (std::string("cudaGraphLaunch: ") + cudaGetErrorString(e)).c_str());
  return GBFFT_OK;
}

int gbfft_batch_destroy(gbfft_batch_t b) {
  if (!b) return GBFFT_OK;
  if (!valid(b)) return set_error(GBFFT_ERR_INVALID, "not a batch");
  drop_graph(b);
  drop_desc(b);
  b->magic = 0;
  delete b;
  return GBFFT_OK;
}

}  // extern "C"
