// ej_join - command-line driver over the C ABI, mirroring the reference's
// standalone executables (e.g. `./HashExe <left> <right>`,
// joins/hashJoin_gpu/main_street/hj.cc:1271-1294): generate the two relations,
// run one join, print the phase timers, the result count and the first three
// result rows (hj.cc:1194-1249).
//
//   ej_join <algo> <left> <right> [--seed N] [--domain D] [--host] [--table R.tbl S.tbl] [--raw R S]
//
// algo: hash | single_hash | bnl | hash_index | sort_index | left_outer.
// left = |S| (probe side), right = |R| (build side), as in the reference.
// Default inputs: R keys a permutation of [0, right), S keys uniform over
// [0, domain) with domain = right (every S row matches exactly once).
// --table reads both relations in the reference's table format (int32 count,
// then TUPLE[count]; joins/hashJoin_gpu/main_street/TableBuild.cpp:118-140),
// --raw as bare TUPLE arrays (the joins/join_ori R and S files); <left> and
// <right> are then ignored.
// --host joins host buffers through ej_join_host (copies inside the timing).
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <string>
#include <vector>

#include "ej.h"

static void die(ej_handle* h, ej_status s, const char* what) {
  fprintf(stderr, "%s: %s %s\n", what, ej_status_name(s), h ? ej_last_error(h) : "");
  exit(1);
}

static std::vector<ej_tuple> read_table(const char* path, ej_table_file_format fmt) {
  uint64_t n = 0;
  ej_status st = ej_table_file_rows(path, fmt, &n);
  std::vector<ej_tuple> t(st == EJ_OK ? (size_t)n : 0);
  if (st == EJ_OK) st = ej_table_file_read(path, fmt, t.data(), n, &n);
  if (st != EJ_OK) {
    fprintf(stderr, "%s: %s\n", path, ej_status_name(st));
    exit(1);
  }
  return t;
}

int main(int argc, char** argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: %s <hash|single_hash|bnl|hash_index|sort_index|left_outer> <left> <right> "
                    "[--seed N] [--domain D] [--host] [--table R.tbl S.tbl] [--raw R S]\n", argv[0]);
    return 2;
  }
  const std::string algo_name = argv[1];
  const char* names[] = {"hash", "single_hash", "bnl", "hash_index", "sort_index", "left_outer"};
  int algo = -1;
  for (int i = 0; i < 6; i++)
    if (algo_name == names[i]) algo = i;
  if (algo < 0) {
    fprintf(stderr, "unknown algorithm %s\n", argv[1]);
    return 2;
  }
  uint64_t left = strtoull(argv[2], nullptr, 10), right = strtoull(argv[3], nullptr, 10);
  uint64_t seed = 1;
  uint32_t domain = (uint32_t)right;
  bool host = false;
  const char* rtab = nullptr;
  const char* stab = nullptr;
  ej_table_file_format tfmt = EJ_TABLE_FILE_COUNTED;
  for (int i = 4; i < argc; i++) {
    if (!strcmp(argv[i], "--seed") && i + 1 < argc) seed = strtoull(argv[++i], nullptr, 10);
    else if (!strcmp(argv[i], "--domain") && i + 1 < argc) domain = (uint32_t)strtoul(argv[++i], nullptr, 10);
    else if (!strcmp(argv[i], "--host")) host = true;
    else if ((!strcmp(argv[i], "--table") || !strcmp(argv[i], "--raw")) && i + 2 < argc) {
      tfmt = !strcmp(argv[i], "--raw") ? EJ_TABLE_FILE_RAW : EJ_TABLE_FILE_COUNTED;
      rtab = argv[++i];
      stab = argv[++i];
    }
  }
  printf("left=%llu:right=%llu\n", (unsigned long long)left, (unsigned long long)right);

  ej_handle* h = nullptr;
  ej_status st = ej_create(0, &h);
  if (st != EJ_OK) die(nullptr, st, "ej_create");
  ej_set_timing(h, 1);

  std::vector<ej_tuple> hR, hS;
  ej_tuple *R = nullptr, *S = nullptr;
  if (rtab) {
    hR = read_table(rtab, tfmt);
    hS = read_table(stab, tfmt);
    right = hR.size();
    left = hS.size();
  }
  if (cudaMalloc(&R, (right ? right : 1) * sizeof(ej_tuple)) != cudaSuccess ||
      cudaMalloc(&S, (left ? left : 1) * sizeof(ej_tuple)) != cudaSuccess) {
    fprintf(stderr, "cudaMalloc failed\n");
    return 1;
  }
  if (rtab) {
    cudaMemcpy(R, hR.data(), right * sizeof(ej_tuple), cudaMemcpyHostToDevice);
    cudaMemcpy(S, hS.data(), left * sizeof(ej_tuple), cudaMemcpyHostToDevice);
  } else {
    if (domain == 0) domain = 1;
    ej_gen_spec rs = {};
    rs.kind = EJ_GEN_PERM;
    rs.n = right;
    rs.domain = right > domain ? (uint32_t)right : domain;
    rs.seed = seed * 2 + 1;
    rs.kseed = seed * 2 + 2;
    rs.dup = 1;
    rs.key_base = 1;  // row ids from 1, like the reference's getTupleId()
    ej_gen_spec ss = {};
    ss.kind = EJ_GEN_UNIFORM;
    ss.n = left;
    ss.domain = domain;
    ss.seed = seed * 2 + 3;
    ss.key_base = (int32_t)(right + 1);
    if ((st = ej_generate(h, &rs, R)) != EJ_OK) die(h, st, "generate R");
    if ((st = ej_generate(h, &ss, S)) != EJ_OK) die(h, st, "generate S");
    if (host) {
      hR.resize(right);
      hS.resize(left);
      cudaMemcpy(hR.data(), R, right * sizeof(ej_tuple), cudaMemcpyDeviceToHost);
      cudaMemcpy(hS.data(), S, left * sizeof(ej_tuple), cudaMemcpyDeviceToHost);
    }
  }

  // count pass sizes the output (the reference's count -> presum -> getValue, hj.cc:997-1069)
  uint64_t count = 0;
  st = ej_join(h, (ej_algo)algo, R, right, S, left, nullptr, 0, &count);
  if (st != EJ_OK && st != EJ_ERR_CAPACITY) die(h, st, "count");
  ej_result* out = nullptr;
  std::vector<ej_result> hout;
  const auto t0 = std::chrono::steady_clock::now();
  if (host) {
    hout.resize(count ? count : 1);
    st = ej_join_host(h, (ej_algo)algo, hR.data(), right, hS.data(), left, hout.data(), count, &count);
  } else {
    if (cudaMalloc(&out, (count ? count : 1) * sizeof(ej_result)) != cudaSuccess) {
      fprintf(stderr, "cudaMalloc of %llu result rows failed\n", (unsigned long long)count);
      return 1;
    }
    st = ej_join(h, (ej_algo)algo, R, right, S, left, out, count, &count);
  }
  const auto t1 = std::chrono::steady_clock::now();
  if (st != EJ_OK) die(h, st, "join");
  float ms[EJ_PHASES];
  ej_last_phase_ms(h, ms);
  const char* phase[EJ_PHASES] = {"build", "partition", "count", "write"};
  for (int i = 0; i < EJ_PHASES; i++) printf("%-10s Diff: %ld us\n", phase[i], (long)(ms[i] * 1000.0f));
  printf("total      Diff: %ld us (host clock%s)\n",
         (long)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count(),
         host ? ", copies included" : "");
  printf("the number of total match tuple = %llu\n", (unsigned long long)count);
  if (!host && count) {
    hout.resize(count < 3 ? count : 3);
    cudaMemcpy(hout.data(), out, hout.size() * sizeof(ej_result), cudaMemcpyDeviceToHost);
  }
  for (size_t i = 0; i < 3 && i < count; i++)
    printf("join[%zu]: rkey=%d rval=%d lkey=%d lval=%d\n", i, hout[i].rkey, hout[i].rval, hout[i].lkey, hout[i].lval);
  cudaFree(out);
  cudaFree(R);
  cudaFree(S);
  ej_destroy(h);
  return 0;
}
