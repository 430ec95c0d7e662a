/*
 * Link stubs for building the MSBG reference library as a CPU oracle.
 * Test infrastructure only.
 *  - libpng/libjpeg are not installed: the two image writers the library
 *    declares (src/bitmap.h:1098-1099, src/bitmap.h:1208-1209) report failure.
 *  - the demo's main.cpp (not built) owns the global thread count that
 *    HaloBlockSet sizes its per-thread buffers by (src/main.cpp:28,
 *    src/msbg.cpp:3095); the driver sets it before any library call.
 */
#include <stdio.h>

int nMaxThreads = -1;

extern "C" {
int BmpWritePNG(FILE *, void *, void *, unsigned) { return -1; }
int BmpSaveBitmapJPG(void *, char *, int, unsigned) { return -1; }
}
