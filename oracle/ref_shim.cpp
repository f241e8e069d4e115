// ref_shim.cpp - feeds seeded relations to the UNMODIFIED reference CPU joins.
//
// TEST INFRASTRUCTURE ONLY (used by oracle/build_ref.sh to make oracle/_ref/*,
// which pin the oracle restatement to the reference's own output).
//
// The reference programs (joins/CPU_JOIN/{hash_cpu,inner_cpu,sortIndex_cpu,
// block_cpu}) generate time-seeded inputs inside createTuple()/init() and take
// no input files.  They are compiled from their own sources with the forced
// include oracle/ref_prelude.h, which renames
//   main -> ej_ref_main   their main() becomes callable from this file
//   free -> ej_ref_free   every free() in their source comes here
// The first free() each of them makes is free(used) at the end of its
// generator (e.g. joins/CPU_JOIN/hash_cpu/hj.cc:102), after the relation
// arrays are allocated and filled: at that moment this file overwrites them
// with the relations read from disk.  When the program frees its result array
// the rows written so far are dumped (the reference only prints a count).
//
// Usage: <prog> <R file> <S file> [dump file]
// R/S files use the reference's table format: int32 count, then TUPLE[count]
// (joins/hashJoin_gpu/main_street/TableBuild.cpp:118-140).  The program is run
// as `<prog> |S| |R|` (left = S = argv[1], right = R = argv[2]).
//
// EJ_REF_TUPLE_BYTES and EJ_REF_ROW_BYTES give the program's TUPLE and result
// row sizes: 8 and 16 for the equi-joins (the default), 32 and 56 for the 3-D
// distance join (joins/CPU_JOIN/3d_cpu/nestLoopJoin.cc:23-33), 24 and 40 for
// the 2-D one (joins/blockJoin_gpu/complex_block/2d_cpu/nestLoopJoin.cc).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifndef EJ_REF_TUPLE_BYTES
#define EJ_REF_TUPLE_BYTES 8
#endif
#ifndef EJ_REF_ROW_BYTES
#define EJ_REF_ROW_BYTES 16
#endif

struct ej_ref_tuple {
  unsigned char bytes[EJ_REF_TUPLE_BYTES];
};

// the reference's globals (unmangled: namespace-scope variables)
extern ej_ref_tuple* EJ_REF_RIGHT;
extern ej_ref_tuple* EJ_REF_LEFT;
#ifdef EJ_REF_RESULT
extern void* EJ_REF_RESULT;
#endif

int ej_ref_main(int argc, char* argv[]);

static ej_ref_tuple* g_right = nullptr;
static ej_ref_tuple* g_left = nullptr;
static int g_nright = 0, g_nleft = 0;
static int g_injected = 0;
static const char* g_dump = nullptr;

static ej_ref_tuple* read_table(const char* path, int* n) {
  FILE* f = fopen(path, "rb");
  if (!f) { perror(path); exit(2); }
  if (fread(n, sizeof(int), 1, f) != 1) { fprintf(stderr, "bad table %s\n", path); exit(2); }
  ej_ref_tuple* t = static_cast<ej_ref_tuple*>(malloc(sizeof(ej_ref_tuple) * (*n > 0 ? *n : 1)));
  if (*n && fread(t, sizeof(ej_ref_tuple), *n, f) != (size_t)*n) { fprintf(stderr, "short table %s\n", path); exit(2); }
  fclose(f);
  return t;
}

extern "C" void ej_ref_free(void* p) {
  if (!g_injected) {
    memcpy(EJ_REF_RIGHT, g_right, sizeof(ej_ref_tuple) * g_nright);
    memcpy(EJ_REF_LEFT, g_left, sizeof(ej_ref_tuple) * g_nleft);
    g_injected = 1;
  }
#ifdef EJ_REF_RESULT
  if (g_dump && p && p == EJ_REF_RESULT) {
    // the result array was calloc'ed, and every row holds a nonzero row id
    // (ids start at 1 in the dumped tables), so the first all-zero row ends
    // the written prefix
    const unsigned char* w = static_cast<const unsigned char*>(p);
    FILE* f = fopen(g_dump, "wb");
    const long max_rows = strtol(getenv("EJ_REF_DUMP_MAX") ? getenv("EJ_REF_DUMP_MAX") : "67108864", nullptr, 10);
    long n = 0;
    for (; n < max_rows; n++) {
      const unsigned char* row = w + (size_t)n * EJ_REF_ROW_BYTES;
      int nonzero = 0;
      for (int b = 0; b < EJ_REF_ROW_BYTES; b++) nonzero |= row[b];
      if (!nonzero) break;
    }
    fwrite(w, EJ_REF_ROW_BYTES, n, f);
    fclose(f);
  }
#endif
  free(p);
}

int main(int argc, char* argv[]) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s <R table> <S table> [dump]\n", argv[0]);
    return 2;
  }
  g_right = read_table(argv[1], &g_nright);
  g_left = read_table(argv[2], &g_nleft);
  g_dump = argc > 3 ? argv[3] : nullptr;
  char a1[32], a2[32];
  snprintf(a1, sizeof a1, "%d", g_nleft);
  snprintf(a2, sizeof a2, "%d", g_nright);
  char* args[] = {argv[0], a1, a2, nullptr};
  return ej_ref_main(3, args);
}
