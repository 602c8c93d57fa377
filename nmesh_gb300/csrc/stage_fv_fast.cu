// stage_fv_fast.cu -- the "fv" finite-volume stage kernels: the code of
// stage_fv.cu built with FMA contraction and one division per WENO
// reconstruction (see the notes at the top of stage_fv.cu).
#define NMG_FV_FAST 1
#include "stage_fv.cu"
