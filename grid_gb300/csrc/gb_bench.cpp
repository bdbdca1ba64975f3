// gb_bench.cpp -- device-timed repetition of one kernel of the path (CUDA events on the
// operator's stream), rotating over several (in, out) field pairs so that the inputs of
// consecutive launches are not the L2-resident outputs of the previous one.
#include <cuda_runtime.h>

#include "gb_ops.h"

using namespace gb;

namespace {
int run_one(Op* op, int which, Field* in, Field* out) {
  switch (which) {
    case 0: in->subset = GB_ODD; return op_dhop_cb(op, in, out, 0);   // DhopEO
    case 1: in->subset = GB_EVEN; return op_dhop_cb(op, in, out, 0);  // DhopOE
    case 2: return op_mooee(op, in, out, 0, nullptr, 0);
    case 3: return op_mooee_inv(op, in, out, 0);
    case 4: return op_meooe5d(op, in, out, 0);
    case 5: in->subset = GB_ODD; return op_mpcdagmpc(op, in, out);
    case 6: return op_dhop_full(op, in, out, 0);
  }
  set_error("bench: unknown kernel %d", which);
  return GB_ERR_BAD_ARG;
}
}  // namespace

extern "C" int gb_bench_kernel(gb_op_t op, int which, gb_field_t* ins, gb_field_t* outs, int n_pairs, int reps,
                               double* ms) {
  if (!op || !ins || !outs || n_pairs < 1 || reps < 1 || !ms) { set_error("bad argument"); return GB_ERR_BAD_ARG; }
  for (int i = 0; i < n_pairs; i++) GB_TRY(run_one(op, which, ins[i], outs[i]));  // warm-up
  cudaEvent_t e0, e1;
  GB_CHECK_CUDA(cudaEventCreate(&e0));
  GB_CHECK_CUDA(cudaEventCreate(&e1));
  GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  GB_CHECK_CUDA(cudaEventRecord(e0, op->stream));
  int rc = GB_OK;
  for (int r = 0; r < reps && rc == GB_OK; r++) rc = run_one(op, which, ins[r % n_pairs], outs[r % n_pairs]);
  GB_CHECK_CUDA(cudaEventRecord(e1, op->stream));
  GB_CHECK_CUDA(cudaEventSynchronize(e1));
  float t = 0;
  GB_CHECK_CUDA(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = double(t) / reps;
  if (rc != GB_OK) return rc;
  return check_device_error(op);
}

extern "C" {

int gb_set_device(int device) {
  GB_CHECK_CUDA(cudaSetDevice(device));
  return GB_OK;
}
int gb_op_sync(gb_op_t op) {
  if (!op) return GB_ERR_BAD_ARG;
  GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  return check_device_error(op);
}
int gb_op_event_record(gb_op_t op, int slot) {
  if (!op || slot < 0 || slot >= 16) { set_error("bad event slot"); return GB_ERR_BAD_ARG; }
  if (!op->events[slot]) GB_CHECK_CUDA(cudaEventCreate(&op->events[slot]));
  GB_CHECK_CUDA(cudaEventRecord(op->events[slot], op->stream));
  return GB_OK;
}
int gb_op_event_elapsed(gb_op_t op, int a, int b, double* ms) {
  if (!op || a < 0 || a >= 16 || b < 0 || b >= 16 || !op->events[a] || !op->events[b] || !ms) {
    set_error("bad event slots");
    return GB_ERR_BAD_ARG;
  }
  GB_CHECK_CUDA(cudaEventSynchronize(op->events[b]));
  float t = 0;
  GB_CHECK_CUDA(cudaEventElapsedTime(&t, op->events[a], op->events[b]));
  *ms = t;
  return GB_OK;
}
int gb_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return GB_ERR_BAD_ARG;
  GB_CHECK_CUDA(cudaMallocHost(ptr, bytes));
  return GB_OK;
}
int gb_host_free(void* ptr) {
  GB_CHECK_CUDA(cudaFreeHost(ptr));
  return GB_OK;
}
int gb_stream_create(void** stream) {
  if (!stream) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  cudaStream_t s = nullptr;
  GB_CHECK_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  *stream = s;
  return GB_OK;
}
int gb_stream_destroy(void* stream) {
  if (stream) GB_CHECK_CUDA(cudaStreamDestroy(static_cast<cudaStream_t>(stream)));
  return GB_OK;
}

}  // extern "C"
