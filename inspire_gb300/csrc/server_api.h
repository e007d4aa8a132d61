// Internal interface of the server object used by the native serving loop
// (serving.cu). Nothing here is part of the public C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

struct inspire_pir_server;

namespace inspire {

struct Workspace;

// `count` consecutive requests laid out back to back in host memory, each
// with first_dim (db_cols words, zero-padded), second_dim, packing_key, and
// the response it receives (l x 2 x d words).
struct RequestSegment {
  int count;
  const void* first_dim;
  const void* second_dim;
  const void* packing_key;
  void* responses;
};

struct ServerGeometry {
  int64_t db_cols;            // words of a zero-padded first dimension
  int64_t interpolated_rows;  // the shortest first dimension accepted
  int d, l, nsd, npk;         // degree, shards, second_dim and key polys
  int word_bytes;             // sizeof(CoeffType)
  bool tensor;                // the tensor-core engine is available
};

ServerGeometry GetGeometry(const inspire_pir_server* s);
// INSPIRE_ENGINE_AUTO -> the engine the server's tuned crossover picks for
// `batch` requests; other engines unchanged.
int ResolveEngine(const inspire_pir_server* s, int engine, int batch);
int64_t BatchWorkspaceBytes(const inspire_pir_server* s, int max_batch);
// A workspace for up to max_batch requests: device buffers, a stream, a
// completion event and, when available, the tensor engine's request planes.
int NewBatchWorkspace(inspire_pir_server* s, int max_batch, Workspace** out,
                      std::string* err);
void DeleteBatchWorkspace(Workspace* w);
// ProcessResponse's request checks that depend on the first dimension only.
int ValidateFirstDim(const inspire_pir_server* s, int64_t first_dim_len,
                     std::string* err);
// Enqueues the copies in, the answer and the copies out of one batch on the
// workspace's stream and records its completion event. Asynchronous.
int LaunchBatch(inspire_pir_server* s, Workspace* w, const RequestSegment* segs,
                int nseg, int engine, std::string* err);
// 1 when the workspace's last batch has finished, 0 while it runs, < 0 on a
// CUDA error.
int QueryBatch(Workspace* w);
// Status of the finished batch (the tensor engine's pipeline flag).
int FinishBatch(inspire_pir_server* s, Workspace* w, int engine,
                std::string* err);

}  // namespace inspire
