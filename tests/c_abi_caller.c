/*
 * A plain C caller of the engine's C ABI (include/vmc_gb300.h), built by tests/test_c_abi_caller.py
 * against the host-emulation build of the library (the same exported symbols; "device" buffers are host
 * memory there).  It does what a C integration does: create a plan, attach a nearest-neighbour
 * Heisenberg operator (bond operator 1/4 [[1,0,0,0],[0,-1,2,0],[0,2,-1,0],[0,0,0,1]] on every bond),
 * size the caller-owned workspace, evaluate amplitudes, log-derivatives and local energies, and write
 * them out for the test to compare with the Python engine.
 *
 *   c_abi_caller R C D chi n tensors.f32 configs.i32 out_prefix
 */
#include <stdio.h>
#include <stdlib.h>

#include "vmc_gb300.h"

static void* read_file(const char* path, size_t* bytes) {
  FILE* f = fopen(path, "rb");
  if (!f) return NULL;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  void* buf = malloc(n > 0 ? (size_t)n : 1);
  if (buf && n > 0 && fread(buf, 1, (size_t)n, f) != (size_t)n) {
    free(buf);
    buf = NULL;
  }
  fclose(f);
  *bytes = (size_t)n;
  return buf;
}

static int write_file(const char* prefix, const char* name, const void* data, size_t bytes) {
  char path[4096];
  snprintf(path, sizeof path, "%s%s", prefix, name);
  FILE* f = fopen(path, "wb");
  if (!f) return 1;
  size_t w = fwrite(data, 1, bytes, f);
  fclose(f);
  return w != bytes;
}

#define CHECK(call)                                                                 \
  do {                                                                              \
    vmc_status st_ = (call);                                                        \
    if (st_ != VMC_OK) {                                                            \
      fprintf(stderr, "%s failed: %d (%s)\n", #call, st_, vmc_status_string(st_)); \
      return 2;                                                                     \
    }                                                                               \
  } while (0)

int main(int argc, char** argv) {
  if (argc != 9) {
    fprintf(stderr, "usage: %s R C D chi n tensors.f32 configs.i32 out_prefix\n", argv[0]);
    return 1;
  }
  const int R = atoi(argv[1]), C = atoi(argv[2]), D = atoi(argv[3]), chi = atoi(argv[4]), n = atoi(argv[5]);
  const int d = 2;
  size_t tbytes = 0, cbytes = 0;
  float* tensors = (float*)read_file(argv[6], &tbytes);
  int32_t* configs = (int32_t*)read_file(argv[7], &cbytes);
  if (!tensors || !configs || cbytes != (size_t)n * R * C * sizeof(int32_t)) {
    fprintf(stderr, "bad inputs\n");
    return 1;
  }

  vmc_shape shape = {R, C};
  vmc_plan* plan = NULL;
  CHECK(vmc_peps_plan(&shape, D, chi, d, VMC_DTYPE_F32, VMC_STRATEGY_ZIP_UP, 2, &plan));

  /* the bond operator on every horizontal and vertical bond; no one-site or diagonal terms */
  const double bond[16] = {0.25, 0, 0, 0, 0, -0.25, 0.5, 0, 0, 0.5, -0.25, 0, 0, 0, 0, 0.25};
  const int n_h = R * (C - 1), n_v = (R - 1) * C;
  double* onesite = (double*)calloc((size_t)R * C * d * d, sizeof(double));
  int* onesite_mask = (int*)calloc((size_t)R * C, sizeof(int));
  double* horiz = (double*)calloc((size_t)(n_h > 0 ? n_h : 1) * 16, sizeof(double));
  int* horiz_mask = (int*)calloc((size_t)(n_h > 0 ? n_h : 1), sizeof(int));
  double* vert = (double*)calloc((size_t)(n_v > 0 ? n_v : 1) * 16, sizeof(double));
  int* vert_mask = (int*)calloc((size_t)(n_v > 0 ? n_v : 1), sizeof(int));
  for (int b = 0; b < n_h; ++b) {
    for (int k = 0; k < 16; ++k) horiz[b * 16 + k] = bond[k];
    horiz_mask[b] = 1;
  }
  for (int b = 0; b < n_v; ++b) {
    for (int k = 0; k < 16; ++k) vert[b * 16 + k] = bond[k];
    vert_mask[b] = 1;
  }
  CHECK(vmc_peps_plan_set_operator(plan, onesite, onesite_mask, horiz, horiz_mask, vert, vert_mask, 0, NULL, NULL,
                                   NULL, NULL, NULL));

  const int64_t np_sliced = vmc_peps_n_params_sliced(plan);
  const size_t ws_bytes = vmc_workspace_size(plan, n);
  void* ws = malloc(ws_bytes ? ws_bytes : 1);
  float* O = (float*)malloc((size_t)n * (size_t)np_sliced * sizeof(float));
  double* logamp = (double*)malloc((size_t)n * sizeof(double));
  double* sign = (double*)malloc((size_t)n * sizeof(double));
  double* E = (double*)malloc((size_t)n * sizeof(double));
  int32_t status = 0;
  CHECK(vmc_peps_amp_grad(plan, NULL, tensors, configs, n, 0, O, logamp, sign, NULL, ws, ws_bytes, &status));
  CHECK(vmc_peps_local_energy(plan, NULL, tensors, configs, n, logamp, sign, E, ws, ws_bytes, &status));
  if (status != 0) {
    fprintf(stderr, "device status %d\n", status);
    return 3;
  }
  int bad = write_file(argv[8], "logamp.f64", logamp, (size_t)n * sizeof(double)) |
            write_file(argv[8], "sign.f64", sign, (size_t)n * sizeof(double)) |
            write_file(argv[8], "E.f64", E, (size_t)n * sizeof(double)) |
            write_file(argv[8], "O.f32", O, (size_t)n * (size_t)np_sliced * sizeof(float));
  printf("%lld %zu\n", (long long)np_sliced, ws_bytes);
  vmc_plan_destroy(plan);
  free(onesite), free(onesite_mask), free(horiz), free(horiz_mask), free(vert), free(vert_mask);
  free(ws), free(O), free(logamp), free(sign), free(E), free(tensors), free(configs);
  return bad ? 4 : 0;
}
