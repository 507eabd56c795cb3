/*
 * nl_prelude.h -- prefix for compiling the kernels of the reference's
 * neighborlist.cu (from its first __global__ to the end of the file) as host
 * C++.  The host functions above them launch kernels with <<<>>> and are not
 * compiled.  The symbols are the ones neighborlist.cu:16-28 declares.
 * TEST INFRASTRUCTURE.
 */
#include "cuda_shim.h"
#include "ref_emu.h"

#define WRAP(x, m) (((x) < m) ? (x) : (x - m))
float rskinsq;
float rmaxdif;
float4 nbox;
float4 nboxi;
int nposit;
int pitch;
unsigned int numTiles;
float4 sharedPos[1024];
float sdata[4096];
