/*
 * inspire_pir.h -- C ABI of the GB300 (sm_103a) ReinsPIRe online answer path.
 *
 * Plain C types only (pointers, sizes, ints): no CUDA, torch or C++ types in
 * any signature, so cgo / JNI / ctypes / N-API bindings can bind it directly.
 * The library is libinspire_gb300.so (built by inspire_gb300/build.py).
 *
 * Every function returns an int status: 0 on success, otherwise the
 * absl::StatusCode the reference would return (3 INVALID_ARGUMENT,
 * 4 DEADLINE_EXCEEDED, 8 RESOURCE_EXHAUSTED, 9 FAILED_PRECONDITION,
 * 13 INTERNAL) with the
 * reference's message text copied into `err` (NUL-terminated, truncated to
 * err_len). `err` may be NULL.
 *
 * Reference interfaces replaced (paths inside google/InsPIRe):
 *   PirServer<Db,Coeff,Mat>::Create          crypto/pir/server/pir_server.h:45-49
 *   PirServer<Db,Coeff,Mat>::ProcessResponse crypto/pir/server/pir_server.h:67-68
 *   PirServer timing getters                  crypto/pir/server/pir_server.h:70-72
 *   Matrix<T>::Multiply                       crypto/matrix.h:86-88, 167-195
 *   Polynomial<T>::InnerProductFft            crypto/polynomial.h:195-199
 *   ExternalProduct                           crypto/external_product.h:29-33
 *   FinalizeMatrixPack                        crypto/lwes_to_rlwe.h:114-121
 */
#ifndef INSPIRE_PIR_H_
#define INSPIRE_PIR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define INSPIRE_OK 0
#define INSPIRE_INVALID_ARGUMENT 3
#define INSPIRE_DEADLINE_EXCEEDED 4
#define INSPIRE_RESOURCE_EXHAUSTED 8
#define INSPIRE_FAILED_PRECONDITION 9
#define INSPIRE_INTERNAL 13

/* Element kinds of a matrix (the reference's DbDataType / MatCoeffType). */
#define INSPIRE_U8 0
#define INSPIRE_U16 1
#define INSPIRE_U32 2
#define INSPIRE_U64 3
#define INSPIRE_I16 4
#define INSPIRE_I32 5

/* Answer engines for the batched entry points. */
#define INSPIRE_ENGINE_PLAIN 0  /* fused CUDA-core GEMV, HBM-bound        */
#define INSPIRE_ENGINE_TENSOR 1 /* 8-bit limbs on the tcgen05 tensor cores */
#define INSPIRE_ENGINE_AUTO 2   /* per batch size: the server's tuned choice */
/* (u16 DB; i16/i32/u32 pack matrices over Z_2^32, i16/i32 over Z_2^64;
 * l*t*d a multiple of 256. Other servers return FAILED_PRECONDITION.) */

/* PirParams<CoeffType> (crypto/pir/pir_params.h:36-105) together with the
 * template arguments of PirServer<DbDataType, CoeffType, MatCoeffType>. */
typedef struct inspire_pir_params {
  int32_t coeff_bits;   /* 8 * sizeof(CoeffType): 32 or 64           */
  int32_t db_kind;      /* DbDataType: INSPIRE_U8 or INSPIRE_U16       */
  int32_t mat_kind;     /* MatCoeffType: INSPIRE_I16, _I32, _U32, _U64 */
  int32_t log_degree;   /* d = 1 << log_degree                         */
  int32_t log_modulus;  /* RlweParams::LogModulus()                    */
  int32_t log_modulus1_after_switch;
  int32_t log_modulus2_after_switch;
  int32_t pack_log_digit;
  int32_t pack_num_digits;
  int32_t eval_log_digit;
  int32_t eval_num_digits;
  int32_t num_entries;
  int32_t interpolation_degree;
  int32_t entry_size_multiple;
  uint64_t plaintext_modulus;
} inspire_pir_params;

typedef struct inspire_pir_server inspire_pir_server;

/*
 * PirServer::Create (crypto/pir/server/pir_server.cc:54-124) from host
 * memory. The material is the server's combined form:
 *   db           (l*t*d) x db_cols matrix of db_kind, row-major (the
 *                vertically concatenated DB matrices; a condensed Matrix has
 *                the same bytes)
 *   pack         (l*t*d) x pack_cols matrix of mat_kind, row-major (the
 *                concatenated PreprocessMatrixPackOutput::matrix, shard-major)
 *   a_tilde_agg  l*t polynomials (shard-major, slice-minor)
 *   t_vec_h      l*t*pack_num_digits polynomials
 *   second_dim_a 2*eval_num_digits polynomials (none when t == 1)
 * Polynomials are d CoeffType words each. Everything is copied to GPU memory
 * once; the host buffers may be freed after the call.
 */
int inspire_pir_server_create(const inspire_pir_params* params,
                              const void* db, int64_t db_rows, int64_t db_cols,
                              const void* pack, int64_t pack_rows,
                              int64_t pack_cols, const void* a_tilde_agg,
                              int64_t a_tilde_agg_count, const void* t_vec_h,
                              int64_t t_vec_h_count, const void* second_dim_a,
                              int64_t second_dim_a_count,
                              inspire_pir_server** out, char* err,
                              size_t err_len);

void inspire_pir_server_destroy(inspire_pir_server* server);

/*
 * PirServer::LoadFromBuffer / LoadFromFile (crypto/pir/server/
 * pir_server.cc:590-791): a server from a SaveToFile image. The DB section
 * is copied from the image straight into GPU memory and the bit-packed pack
 * matrix is unpacked on the GPU. Truncated images give INTERNAL "Error
 * reading from buffer"; an unreadable file "Failed to read file.".
 */
int inspire_pir_server_load(const inspire_pir_params* params,
                            const void* buffer, size_t size,
                            inspire_pir_server** out, char* err,
                            size_t err_len);
int inspire_pir_server_load_file(const inspire_pir_params* params,
                                 const char* path, inspire_pir_server** out,
                                 char* err, size_t err_len);

/*
 * PirServer::SaveToFile (crypto/pir/server/pir_server.cc:434-588): the
 * server's image, byte-compatible with the reference's loader. With buffer
 * NULL (or too small: RESOURCE_EXHAUSTED) *size receives the image size.
 * A server loaded from an image saves the same bytes.
 */
int inspire_pir_server_save(inspire_pir_server* server, void* buffer,
                            size_t capacity, size_t* size, char* err,
                            size_t err_len);
int inspire_pir_server_save_file(inspire_pir_server* server, const char* path,
                                 char* err, size_t err_len);

/*
 * PirServer::ProcessResponse (crypto/pir/server/pir_server.cc:154-306) for
 * one request in host memory. first_dim has first_dim_len CoeffType words,
 * second_dim second_dim_count polynomials, packing_key packing_key_count
 * polynomials. response receives l ciphertexts, each a then b (2*l*d
 * words). Synchronous; updates the timers.
 */
int inspire_pir_process_response(inspire_pir_server* server,
                                 const void* first_dim, int64_t first_dim_len,
                                 const void* second_dim,
                                 int64_t second_dim_count,
                                 const void* packing_key,
                                 int64_t packing_key_count, void* response,
                                 char* err, size_t err_len);

/*
 * ProcessResponse for `batch` requests in host memory, stacked: request q's
 * first_dim starts at q*first_dim_len words, its second_dim at
 * q*second_dim_count*d, its packing key at q*packing_key_count*d; responses
 * are stacked the same way (2*l*d words each). `engine` selects the DB/pack
 * product (INSPIRE_ENGINE_*); responses are identical for every engine.
 */
int inspire_pir_process_batch(inspire_pir_server* server, int32_t batch,
                              const void* first_dim, int64_t first_dim_len,
                              const void* second_dim, int64_t second_dim_count,
                              const void* packing_key,
                              int64_t packing_key_count, void* responses,
                              int32_t engine, char* err, size_t err_len);

/*
 * Device-resident form of inspire_pir_process_batch: all pointers are CUDA
 * device pointers and the work is enqueued on `stream` (a cudaStream_t, or
 * NULL for the legacy default stream) without synchronising. first_dim holds
 * first_dim_len words per request; when that is below db_cols the library
 * copies the batch into its workspace and zero-pads it there.
 */
int inspire_pir_process_batch_device(inspire_pir_server* server,
                                     int32_t batch, const void* first_dim,
                                     int64_t first_dim_len,
                                     const void* second_dim,
                                     int64_t second_dim_count,
                                     const void* packing_key,
                                     int64_t packing_key_count,
                                     void* responses, int32_t engine,
                                     void* stream, char* err, size_t err_len);

/*
 * Stage 1 alone for a device-resident batch: out[q][r] = (DB * q1_q)[r] +
 * (P * y_g,q)[r], the b' + b_agg_partial vector that FinalizeMatrixPack
 * consumes (pir_server.cc:215-254), exact in the bits the answer reads:
 * mod 2^w with the plain engine and for Z_2^32; a Z_2^64 server with
 * log_modulus <= 56 on the tensor engine computes the words mod 2^56 only
 * (the top digit position's products reach no lower bit, and
 * FinalizeMatrixPack keeps LowBits(., log_modulus), lwes_to_rlwe.cc:464-469).
 * first_dim holds db_cols words per request, packing_key 2*pack_num_digits
 * polynomials per request (its first half is y_vec_g); out holds rows words
 * per request. Enqueued on `stream` without synchronising.
 */
int inspire_pir_products_device(inspire_pir_server* server, int32_t batch,
                                const void* first_dim, const void* packing_key,
                                void* out, int32_t engine, void* stream,
                                char* err, size_t err_len);

/*
 * Stage 1 of a device-resident batch on the tensor engine in a given form
 * (no reference counterpart: the forms are this build's layouts and tile
 * shapes of the same product). form INSPIRE_FORM_PLANES reads the DB as
 * resident fp16 digit planes, INSPIRE_FORM_RAW reads the DB as stored (u16)
 * and splits it into digits in shared memory; or-ed with
 * INSPIRE_FORM_NARROW the kernel takes 16 requests per tile instead of 64.
 * The raw form and the narrow tiles serve Z_2^32 servers; a Z_2^64 server
 * runs the planes with 32-request tiles. split > 0 forces that split-K factor (0: the tuned or
 * heuristic one). Same buffers as inspire_pir_products_device with
 * INSPIRE_ENGINE_TENSOR; the words are exact mod 2^w in every case (all
 * digit positions computed). FAILED_PRECONDITION when the server has no
 * such form.
 */
#define INSPIRE_FORM_PLANES 0
#define INSPIRE_FORM_RAW 1
#define INSPIRE_FORM_NARROW 2
int inspire_pir_tensor_products_device(inspire_pir_server* server,
                                       int32_t batch, const void* first_dim,
                                       const void* packing_key, void* out,
                                       int32_t form, int32_t split,
                                       void* stream, char* err,
                                       size_t err_len);

/*
 * The packing step of a device-resident batch, as the packing benchmark's
 * server loop runs it (crypto/pir/benchmarking/pir_packing_metrics_tool.cc:
 * 226-283): DB * q1 + P * y_g, then FinalizeMatrixPack
 * (crypto/lwes_to_rlwe.cc:448-479) of every shard, with no EvalPoly and no
 * modulus switch. out: batch x (l*t) x 2 x d words, the (a_tilde_agg, b_agg)
 * pair of each shard. Same validation and error strings as ProcessResponse;
 * enqueued on `stream` without synchronising.
 */
int inspire_pir_pack_batch_device(inspire_pir_server* server, int32_t batch,
                                  const void* first_dim, int64_t first_dim_len,
                                  const void* packing_key,
                                  int64_t packing_key_count, void* out,
                                  int32_t engine, void* stream, char* err,
                                  size_t err_len);

/*
 * ExternalProduct (crypto/external_product.cc:35-114) of `batch` independent
 * RLWE ciphertexts, each with its own RGSW ciphertext, under the server's
 * eval gadget (eval_log_digit x eval_num_digits, log_modulus). Device
 * pointers: ct = batch x 2 x d words (a, b); rgsw = batch x 2*ne x 2 x d
 * (u[0..ne) then v[0..ne), each an (a, b) pair, the layout
 * inspire_external_product takes); out = batch x 2 x d. Enqueued on `stream`.
 */
int inspire_pir_external_product_device(inspire_pir_server* server,
                                        int32_t batch, const void* ct,
                                        const void* rgsw, void* out,
                                        void* stream, char* err,
                                        size_t err_len);

/*
 * CUDA graphs of the device entry points (no reference counterpart: the
 * reference has no GPU). inspire_graph_begin starts capturing `stream` (a
 * created stream, not the legacy default one); the device calls made on it
 * by this thread are recorded, not run; inspire_graph_end instantiates them
 * and inspire_graph_launch replays them, with the same pointers and batch
 * sizes, as one launch. Make each call once outside a capture first, with
 * the same batch sizes: that allocates the workspace and request planes
 * (allocation inside a capture fails the capture). The recorded calls use
 * the server's own workspace, so a replay must not overlap any other call
 * on that server. inspire_pir_server_check reports a tensor-engine pipeline
 * timeout recorded by earlier launches (call it after synchronising).
 */
/*
 * Autotuner of the tensor engine (no reference counterpart): times the
 * batched product for `batch` requests on this server's matrices in every
 * available form (resident digit planes or the DB as stored), request tile
 * (64 requests, 32 over Z_2^64; or 16, tried up to 64 requests) and split-K
 * factor, and keeps the fastest for later batches of the same size
 * (rounded up to 16 requests). Reports the split-K factor and the product's
 * time in ms. Synchronous; FAILED_PRECONDITION without the tensor engine.
 */
int inspire_pir_autotune(inspire_pir_server* server, int32_t batch,
                         int32_t* split, float* ms, char* err, size_t err_len);

/*
 * Engine autotuner (no reference counterpart): times the plain engine and
 * the tensor engine (every form and split-K factor, as inspire_pir_autotune)
 * on this server's matrices at batch sizes 1..8, the powers of two up to
 * max_batch and max_batch itself, and keeps as the server's crossover the
 * smallest tested size from which the tensor engine is faster at every
 * larger tested size (0x7fffffff: never, or no tensor engine). Calls with
 * INSPIRE_ENGINE_AUTO then use the tensor engine for batches of at least
 * the crossover (5 until this has run). Synchronous.
 */
int inspire_pir_tune_engines(inspire_pir_server* server, int32_t max_batch,
                             int32_t* crossover, char* err, size_t err_len);

/*
 * The measurements of the last inspire_pir_tune_engines call (no reference
 * counterpart): per tested batch size, the plain and the tensor engine's
 * product time (ms), and the tensor engine's chosen form (INSPIRE_FORM_*,
 * with INSPIRE_FORM_NARROW) and split-K factor. Fills up to `cap` rows of
 * the non-null arrays and returns the number of rows (0 before any tuning,
 * -1 for a null server).
 */
int32_t inspire_pir_engine_table(inspire_pir_server* server, int32_t cap,
                                 int32_t* batch, float* plain_ms,
                                 float* tensor_ms, int32_t* form,
                                 int32_t* split);

typedef struct inspire_graph inspire_graph;
int inspire_graph_begin(void* stream, char* err, size_t err_len);
int inspire_graph_end(void* stream, inspire_graph** out, char* err,
                      size_t err_len);
int inspire_graph_launch(inspire_graph* graph, void* stream, char* err,
                         size_t err_len);
void inspire_graph_destroy(inspire_graph* graph);
int inspire_pir_server_check(inspire_pir_server* server, char* err,
                             size_t err_len);

/*
 * Resident layout of the tensor engine (no reference counterpart). With
 * keep != 0 (the default after create / load) the server keeps the DB's
 * fp16 digit planes resident beside the DB (twice the DB's bytes): the
 * fastest form for large batches. With keep == 0 it drops them and the
 * tensor engine reads the u16 DB as stored, splitting it into digits in
 * shared memory (the DB then takes its own bytes only; large batches run
 * slower, small ones as fast or faster). Re-creates the engine and clears
 * the tuned choices; synchronises the device. Call it between batches,
 * never while a call on this server is in flight. INTERNAL if the engine
 * cannot be re-created (the server then answers with the plain engine).
 */
int inspire_pir_server_set_tensor_planes(inspire_pir_server* server,
                                         int32_t keep, char* err,
                                         size_t err_len);

/*
 * Device bytes the server holds resident: the DB and pack matrices plus the
 * tensor engine's digit planes (workspaces not included). -1 for a null
 * server. No reference counterpart.
 */
int64_t inspire_pir_server_device_bytes(const inspire_pir_server* server);

/*
 * VpirServer::ProcessResponse (crypto/vpir/server/vpir_server.cc:102-195)
 * for `batch` requests in host memory, on a server created with
 * interpolation_degree 1 and entry_size_multiple = ell (DB: ell*d rows x N
 * columns): b' = DB * q1 and b_agg_partial = P * y_g, then per shard
 * LowBits(b' + b_agg_partial) when local_finalize, else FinalizeMatrixPack's
 * b. first_dim: N words per request (the flattened first-dimension
 * polynomials); packing_key: pack_num_digits polynomials per request when
 * local_finalize, else 2*pack_num_digits. b_responses: ell*d words per
 * request (the VpirResponse b polynomials). The reference's messages:
 * "Packing key must contain K polynomials.", "Flattened first dimension
 * query must match DB matrix columns (N).".
 */
int inspire_vpir_process_batch(inspire_pir_server* server, int32_t batch,
                               const void* first_dim, int64_t first_dim_len,
                               const void* packing_key,
                               int64_t packing_key_count,
                               int32_t local_finalize, void* b_responses,
                               int32_t engine, char* err, size_t err_len);

/*
 * Workspaces: the state of one in-flight batch (device buffers, the tensor
 * engine's request byte planes, a CUDA stream, pinned host staging). Several
 * workspaces of one server run concurrently on their own streams; this is
 * what a continuous-batching request loop submits to. A workspace is used
 * by one thread at a time.
 */
typedef struct inspire_pir_workspace inspire_pir_workspace;

/* Device bytes one workspace of max_batch requests holds (HBM admission). */
int64_t inspire_pir_workspace_bytes(const inspire_pir_server* server,
                                    int32_t max_batch);

int inspire_pir_workspace_create(inspire_pir_server* server, int32_t max_batch,
                                 inspire_pir_workspace** out, char* err,
                                 size_t err_len);

void inspire_pir_workspace_destroy(inspire_pir_workspace* ws);

/* Pinned host staging of a workspace, max_batch requests each: first_dim
 * holds db_cols words per request (zero past first_dim_len), second_dim
 * 2*eval_num_digits polynomials, packing_key 2*pack_num_digits polynomials,
 * responses 2*l polynomials. */
int inspire_pir_workspace_host_buffers(inspire_pir_workspace* ws,
                                       void** first_dim, void** second_dim,
                                       void** packing_key, void** responses);

/* Enqueues ProcessResponse for the first `batch` staged requests (copies in,
 * answer, copies the responses back to the staging) and returns at once. */
int inspire_pir_workspace_submit(inspire_pir_workspace* ws, int32_t batch,
                                 int32_t engine, char* err, size_t err_len);

/* 1 when the last submitted batch has finished, 0 while it runs, < 0 on a
 * CUDA error. */
int inspire_pir_workspace_poll(inspire_pir_workspace* ws);

/* Blocks until the last submitted batch has finished; its status. */
int inspire_pir_workspace_wait(inspire_pir_workspace* ws, char* err,
                               size_t err_len);

/*
 * Continuous batching (no reference counterpart: the reference answers one
 * request per ProcessResponse call). One engine serves several servers
 * ("queues", which may differ in ring degree, interpolation degree and entry
 * size multiple). Each queue owns a ring of `ring_slots` request slots in
 * pinned host memory; a scheduler thread batches the submitted slots of a
 * queue in ring order (up to max_batch per batch) onto the queue's in-flight
 * workspaces as soon as one is free, so batches of all queues overlap on the
 * device. Workspaces per queue: hbm_budget / n_servers / the workspace bytes
 * of max_batch requests, between 1 and max_workspaces. Batches of more than
 * plain_max_batch requests use the tensor engine when the server has it.
 * max_wait_us is the batching window: a queue's partial batch waits until its
 * oldest request has waited that long (0: launch as soon as a workspace is
 * free, the lowest latency at light load).
 * Every response is the one inspire_pir_process_response gives for the same
 * request.
 *
 * A caller: inspire_serving_acquire (a slot: pointers to its first_dim
 * (db_cols words), second_dim (2*ne*d), packing_key (2*k*d) and response
 * (l*2*d) areas) -> writes the request -> inspire_serving_submit (with the
 * first dimension's length; the rest of the slot's first_dim is zeroed;
 * ProcessResponse's checks and messages) -> inspire_serving_wait -> reads
 * the response -> inspire_serving_release. A slot is written by its caller
 * only between acquire and submit. Destroy the engine after the last wait
 * has returned; requests still queued then are dropped.
 */
typedef struct inspire_serving inspire_serving;

typedef struct inspire_serving_stats {
  int64_t requests;        /* completed since the last reset */
  int64_t failed;
  int64_t batches;
  int64_t tensor_batches;
  double mean_batch;
  double p50_ms;           /* submit -> completion, over completed requests */
  double p99_ms;
  double max_ms;
  int32_t max_inflight;    /* batches on the device at once, all queues */
  int32_t reserved;
} inspire_serving_stats;

int inspire_serving_create(inspire_pir_server* const* servers,
                           int32_t n_servers, int32_t max_batch,
                           int32_t plain_max_batch, int32_t max_wait_us,
                           int32_t ring_slots, int64_t hbm_budget,
                           int32_t max_workspaces, inspire_serving** out,
                           char* err, size_t err_len);
/* The same scheduler over a host-only loopback device (for tests on machines
 * without a GPU): queue q has slots of slot_words[4q..4q+3] u32 words
 * (first_dim, second_dim, packing_key, response); response word k is
 * first_dim[0] * 7 + q + k, ready delay_us after the batch launches; a
 * request whose first word is 0xDEAD fails its batch. */
int inspire_serving_create_loopback(int32_t n_queues, const int64_t* slot_words,
                                    int32_t workspaces, int32_t delay_us,
                                    int32_t max_batch, int32_t plain_max_batch,
                                    int32_t max_wait_us, int32_t ring_slots,
                                    inspire_serving** out, char* err,
                                    size_t err_len);
void inspire_serving_destroy(inspire_serving* engine);
/* Blocks up to timeout_ms for a free slot (RESOURCE_EXHAUSTED after). */
int inspire_serving_acquire(inspire_serving* engine, int32_t queue,
                            int32_t timeout_ms, int64_t* ticket,
                            void** first_dim, void** second_dim,
                            void** packing_key, void** response, char* err,
                            size_t err_len);
int inspire_serving_submit(inspire_serving* engine, int64_t ticket,
                           int64_t first_dim_len, char* err, size_t err_len);
/* 0 when the response is in the slot; the request's error status otherwise;
 * DEADLINE_EXCEEDED if still running after timeout_ms. */
int inspire_serving_wait(inspire_serving* engine, int64_t ticket,
                         int32_t timeout_ms, char* err, size_t err_len);
int inspire_serving_release(inspire_serving* engine, int64_t ticket);
int inspire_serving_get_stats(inspire_serving* engine,
                               inspire_serving_stats* out);
int inspire_serving_reset_stats(inspire_serving* engine);
int inspire_serving_queue_info(inspire_serving* engine, int32_t queue,
                               int32_t* workspaces, int64_t* workspace_bytes,
                               int32_t* ring_slots);

/* Server geometry: rows = l*t*d, and the column counts of both matrices. */
int inspire_pir_server_shape(const inspire_pir_server* server, int64_t* rows,
                             int64_t* db_cols, int64_t* pack_cols);

/* GetDbMultiplyTime / GetPackingTime / GetPolyEvalTime
 * (crypto/pir/server/pir_server.h:70-72), accumulated in milliseconds. */
int inspire_pir_server_timings(const inspire_pir_server* server,
                               double* db_mult_ms, double* packing_ms,
                               double* poly_eval_ms);

/* ---- Component entry points (host memory in and out, synchronous) ---- */

/* Matrix<mat_kind>::Multiply<CoeffType> (crypto/matrix.h:167-195):
 * out[r] = sum_c mat[r][c] * vec[c] mod 2^coeff_bits. */
int inspire_matrix_multiply(int32_t mat_kind, int32_t coeff_bits,
                            const void* mat, int64_t rows, int64_t cols,
                            const void* vec, void* out, char* err,
                            size_t err_len);

/* Polynomial<T>::InnerProductFft (crypto/polynomial_fft.cc:68-197): the
 * exact value sum_i u_i * v_i in Z_{2^w}[X]/(X^d+1) for the operands that
 * its chunk rule (u_bits, v_bits, chunk_bits, u_is_signed) reads. */
int inspire_inner_product(int32_t coeff_bits, const void* u, const void* v,
                          int32_t n, int32_t d, int32_t u_bits, int32_t v_bits,
                          int32_t chunk_bits, int32_t u_is_signed, void* out,
                          char* err, size_t err_len);

/* ExternalProduct (crypto/external_product.cc:35-114). rgsw holds
 * u[0..nd) then v[0..nd), each an (a, b) pair of polynomials. */
int inspire_external_product(const inspire_pir_params* params,
                             const void* ct_a, const void* ct_b,
                             const void* rgsw, void* out_a, void* out_b,
                             char* err, size_t err_len);

/* FinalizeMatrixPack (crypto/lwes_to_rlwe.cc:448-479): the b polynomial of
 * the packed ciphertext (its a polynomial is a_tilde_agg unchanged). */
int inspire_finalize_matrix_pack(const inspire_pir_params* params,
                                 const void* b, const void* b_agg_partial,
                                 const void* y_vec_h, const void* t_vec_h,
                                 void* out_b, char* err, size_t err_len);

/*
 * Offline DB preparation: PreprocessingServer::Preprocess's interpolation
 * and transposition for every shard (crypto/pir/server/
 * preprocessing_server.h:68-95, 174-209) on the GPU. db_raw holds
 * num_entries records of entry_size_multiple * ring_degree values
 * (value_bits = 8, 16 or 32), record-major as Preprocess takes it;
 * db_raw_len counts values. out receives the combined DB matrix of
 * l*t*d rows and out_cols columns (>= num_entries / t; columns past it are
 * zeroed, the padding Preprocess adds for u64 coefficients), row-major:
 * row k*t*d + j*d + c, column i = coefficient c of the j-th interpolated
 * polynomial of records i*t .. i*t+t-1 in shard k (Interpolate,
 * crypto/db_row_interpolation.cc:115-228). on_device = 1: device pointers,
 * enqueued on `stream`; 0: host pointers, synchronous. Errors carry the
 * reference's messages ("Invalid raw database size.", "ring_degree must be
 * a power of two.", ...).
 */
int inspire_interpolate_db(int32_t value_bits, const void* db_raw,
                           int64_t db_raw_len, int64_t num_entries,
                           int32_t ring_degree, int32_t interpolation_degree,
                           int32_t entry_size_multiple,
                           uint32_t plaintext_modulus, void* out,
                           int64_t out_cols, int32_t on_device, void* stream,
                           char* err, size_t err_len);

/*
 * ComputeHintMatrix (crypto/hint_computation.cc:78-160) on the GPU: for a
 * database of `rows` x `cols` entries (db_kind = INSPIRE_U8, _U16 or _U32)
 * and n a-components of d CoeffType coefficients (cols = n * d), row i of
 * the rows x d result is sum_k (row i's k-th block of d entries) times the
 * negacyclic matrix of a_k, mod 2^coeff_bits (the reference's naive
 * definition, hint_computation_test.cc:36-176), computed exactly with
 * multi-prime NTTs. on_device = 1: device pointers on `stream`; 0: host
 * pointers. The reference's error messages.
 */
int inspire_compute_hint_matrix(int32_t db_kind, int32_t coeff_bits,
                                const void* db, int64_t rows, int64_t cols,
                                const void* a_components, int32_t n,
                                int32_t d, void* out, int32_t on_device,
                                void* stream, char* err, size_t err_len);

/*
 * PreprocessMatrixPack (crypto/lwes_to_rlwe.cc:414-446, called per slice by
 * PreprocessingServer::ComputePreprocessedOutputs,
 * crypto/pir/server/preprocessing_server.h:248-271) for `slices` slices at
 * once, exact (multi-prime NTT products, integer transforms):
 *   hint    : slices*d rows of >= d CoeffType words, row stride hint_stride
 *             (the hint matrix; slice i reads rows i*d .. i*d+d-1, columns
 *             0..d-1, as its d LWE a-vectors)
 *   pack_a  : 2*num_digits polynomials: w_vec_g then w_vec_h
 *   a_tilde_agg : slices x d words;  t_vec_h : slices x num_digits x d words
 *   matrix  : (slices*d) x (num_digits*d) entries of mat_kind (the
 *             coefficient type, INSPIRE_I16 or INSPIRE_I32): the slices'
 *             matrices stacked, i.e. the server's pack matrix
 * on_device = 1: device pointers, work on `stream`; 0: host pointers.
 */
int inspire_preprocess_matrix_pack(int32_t coeff_bits, int32_t mat_kind,
                                   int32_t log_modulus, int32_t log_digit,
                                   int32_t num_digits, int32_t d, int32_t slices,
                                   const void* hint, int64_t hint_stride,
                                   const void* pack_a, int64_t pack_a_count,
                                   void* a_tilde_agg, void* matrix, void* t_vec_h,
                                   int32_t on_device, void* stream, char* err,
                                   size_t err_len);

/*
 * PirPreprocessedData in its protobuf form (crypto/proto/pir_server.proto):
 * DeserializePirPreprocessedData + PirServer::Create straight to GPU memory
 * (the contents LoadPirPreprocessedDataFromFile reads,
 * crypto/pir/server/pir_preprocessed_data.h:96-139), the directory form
 * (metadata.bin + shard_<i>.bin, LoadPirPreprocessedDataFromDirectory,
 * :203-267), and the reverse (SerializePirPreprocessedData,
 * SavePirPreprocessedDataToDirectory). save: with buffer == NULL only *size
 * is set. The reference's parse / size error messages.
 */
int inspire_pir_server_load_preprocessed(const inspire_pir_params* params,
                                         const void* buffer, size_t size,
                                         inspire_pir_server** out, char* err,
                                         size_t err_len);
int inspire_pir_server_load_preprocessed_dir(const inspire_pir_params* params,
                                             const char* dir,
                                             inspire_pir_server** out,
                                             char* err, size_t err_len);
int inspire_pir_server_save_preprocessed(inspire_pir_server* server,
                                         void* buffer, size_t capacity,
                                         size_t* size, char* err,
                                         size_t err_len);
int inspire_pir_server_save_preprocessed_dir(inspire_pir_server* server,
                                             const char* dir, char* err,
                                             size_t err_len);

/*
 * A batched PIR client on the GPU, for load generation and end-to-end tests
 * (PirClient, crypto/pir/client/pir_client.cc:61-272). Client b holds the
 * ternary secret key secret_keys[b][0..d) (values -1, 0, 1) and asks for
 * entry indices[b]. a_components are the public a-components the server was
 * preprocessed with, in PreprocessingServer::Preprocess's order
 * (preprocessing_server.h:96-112): NumFirstDimSamples first-dimension ones,
 * 2*eval_num_digits second-dimension ones when t > 1, 2*pack_num_digits
 * packing ones. Errors are centred binomials of `variance` from a
 * counter-based hash of (seed, client, row, coefficient): reproducible, NOT
 * cryptographically secure (the reference samples with ChaCha). Outputs per
 * client: first_dim[n/t], second_dim[2*ne][d] (absent when t == 1),
 * packing_key[2*k][d], CoeffType words. "Index out of bounds." for a bad
 * index. on_device = 1: device pointers on `stream`; 0: host pointers.
 */
int inspire_client_create_requests(const inspire_pir_params* params,
                                   const int8_t* secret_keys,
                                   const void* a_components, int64_t a_count,
                                   const int64_t* indices, int32_t batch,
                                   uint64_t seed, int32_t variance,
                                   void* first_dim, void* second_dim,
                                   void* packing_key, int32_t on_device,
                                   void* stream, char* err, size_t err_len);

/* PirClient::ProcessResponse (DecryptAfterModulusSwitch per ciphertext,
 * crypto/encryption.cc:330-376) for a batch: responses[b] holds
 * entry_size_multiple ciphertexts (a then b, d words each); out[b] the
 * entry_size_multiple*d plaintext words. */
int inspire_client_process_responses(const inspire_pir_params* params,
                                     const int8_t* secret_keys,
                                     const void* responses, int32_t batch,
                                     void* out, int32_t on_device, void* stream,
                                     char* err, size_t err_len);

/* Interpolate (crypto/db_row_interpolation.h) of one row of t*d values,
 * host pointers: out[j*d + c] = coefficient c of polynomial j. */
int inspire_interpolate(int32_t value_bits, const void* db_row,
                        int64_t db_row_len, int32_t ring_degree,
                        int32_t interpolation_degree,
                        uint32_t plaintext_modulus, void* out, char* err,
                        size_t err_len);

/*
 * InnerProductFft that allocates no GPU memory, for callers that cannot call
 * cudaMalloc (a host runtime that owns the device memory budget, a request
 * path that must not block on allocation). No counterpart in the reference:
 * it computes exactly what inspire_inner_product computes, but u, v and out
 * are device pointers owned by the caller (n*d, n*d and d CoeffType words),
 * the work is enqueued on `stream` (a cudaStream_t, or NULL) without
 * synchronising, and the NTT scratch is a fixed 1.6 MB __device__ array
 * inside the library. Limits: n <= 8 polynomials, d <= 4096; larger sizes are
 * rejected with INVALID_ARGUMENT. The first call on each device looks up that
 * array's device address (cudaGetSymbolAddress), so make the first call on a
 * device before capturing any stream. All calls share the array: calls whose
 * GPU work overlaps (different streams or threads) race and must be
 * serialised by the caller.
 */
int inspire_inner_product_noalloc(int32_t coeff_bits, const void* u,
                                  const void* v, int32_t n, int32_t d,
                                  int32_t u_bits, int32_t v_bits,
                                  int32_t chunk_bits, int32_t u_is_signed,
                                  void* out, void* stream, char* err,
                                  size_t err_len);

#ifdef __cplusplus
}
#endif

#endif /* INSPIRE_PIR_H_ */
