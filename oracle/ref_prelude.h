/* ref_prelude.h - forced include (-include) for compiling a reference CPU join
 * program against oracle/ref_shim.cpp.  TEST INFRASTRUCTURE ONLY.
 * The standard headers come first so their own declarations keep the real
 * names; the reference source that follows sees main() and free() renamed. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <cstdlib>
#include <cstdio>
extern "C" void ej_ref_free(void* p);
#define free ej_ref_free
#define main ej_ref_main
