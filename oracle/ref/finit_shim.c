/* finit_shim.c -- test-side stand-in for the reference's finit()
   (src/main/main/utilities.c:291, a bit-level finiteness test), so that the
   reference's newton1d_brak.c can be compiled on its own into
   oracle/_ref/libnewton1d.so (see Makefile target newton). */
#include <math.h>

int finit(double x) { return isfinite(x) ? 1 : 0; }
