/*
 * ref_emu.h -- entry points of the CPU-emulated reference kernels.
 * TEST INFRASTRUCTURE (golden-vector generation only).
 */
#ifndef REF_EMU_H
#define REF_EMU_H

#include <functional>
#include <vector_types.h>

void emu_launch(unsigned grid, unsigned block, const std::function<void()> &body);

/* Values of the reference's __constant__ symbols (forces.cu:37-64,
 * integrator.cu:28-38, neighborlist.cu:18-25). */
struct RefConsts {
    int natom, ntype, pitch;
    float4 box, boxi;
    float rcutsq, reacf;
    float lj1[64], lj2[64];
    float palfa, alfasq, spiialfa, wolf;
    float bnd1[8], bnd2[8], ang1[8], ang2[8];
    float dt, temper_0;
    unsigned nblocks;
    float rskinsq, rmaxdif;
};

void ref_set_consts(const RefConsts &c, const float4 *pos);

/* one launch each, grid = pitch/256 blocks of 256 threads unless noted */
void ref_nlist_nsquared(float4 *pos, float4 *pos_old, unsigned *nnlist, unsigned *nnlist_max, uint4 *excl);
int ref_nlist_check(float4 *pos, float4 *pos_old);
void ref_pair(int kind, float4 *force, unsigned *nnlist, unsigned *nnlist_max);
void ref_bonds(float4 *force, uint2 *bndlist, unsigned *bndlist_max);
void ref_angles(float4 *force, uint4 *anglist, unsigned *anglist_max);
void ref_leapfrog_nve(float4 *pos, float4 *vel, float4 *force);
void ref_leapfrog_nvt(float4 *pos, float4 *vel, float4 *force, float scale, float *ke_sum);
void ref_ke_sum(float *ke_sum);   /* one block of nblocks threads */
void ref_vv_pre(float4 *pos, float4 *vel, float4 *force);
void ref_vv_cor(float4 *vel, float4 *force);

#endif
