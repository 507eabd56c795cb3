/*
 * ref_kernels.cpp -- compiles the reference's kernel files unchanged, as host
 * C++ through cuda_shim.h, and wraps each kernel in an emulated launch.
 * TEST INFRASTRUCTURE.  The symbols below are the __constant__ variables the
 * reference declares in forces.cu:37-64 and integrator.cu:28-38 (the files
 * that #include the kernel files); their initialisers repeat the reference's
 * published constants (A&S 7.1.26 coefficients, the Coulomb factor).
 */
#include "cuda_shim.h"
#include "ref_emu.h"

int natoms;
int ntype;
float4 fbox;
float4 fboxi;
int pitch_f;
float rcutsq;
float reacf;
float qfac = 1389.35427611722f;
float lj1[64];
float lj2[64];
float a1 = 0.254829592f;
float a2 = -0.284496736f;
float a3 = 1.421413741f;
float a4 = -1.453152027f;
float a5 = 1.061405429f;
float palfa;
float alfasq;
float spiialfa;
float wolf;
float bnd1[8];
float bnd2[8];
float ang1[8];
float ang2[8];
texture<float4, 1, cudaReadModeElementType> posTex;

float4 box;
float4 boxi;
int natom;
float dt;
unsigned int enstype;
float temper_0;
float tcons;
float press_0;
float pcons;
unsigned int nblocks;

float Ke_shared[8192];

#include "pair_forces.cu"
#include "bonded_forces.cu"
#include "nve_leapfrog.cu"
#include "nvt_leapfrog_ber.cu"
#include "nve_vverlet.cu"

void ref_nl_set_consts(const RefConsts &c);

void ref_set_consts(const RefConsts &c, const float4 *pos)
{
    natoms = c.natom; natom = c.natom; ntype = c.ntype; pitch_f = c.pitch;
    fbox = c.box; fboxi = c.boxi; box = c.box; boxi = c.boxi;
    rcutsq = c.rcutsq; reacf = c.reacf;
    for (int i = 0; i < 64; i++) { lj1[i] = c.lj1[i]; lj2[i] = c.lj2[i]; }
    palfa = c.palfa; alfasq = c.alfasq; spiialfa = c.spiialfa; wolf = c.wolf;
    for (int i = 0; i < 8; i++) { bnd1[i] = c.bnd1[i]; bnd2[i] = c.bnd2[i]; ang1[i] = c.ang1[i]; ang2[i] = c.ang2[i]; }
    dt = c.dt; temper_0 = c.temper_0; nblocks = c.nblocks;
    posTex.ptr = pos;
    ref_nl_set_consts(c);
}

static unsigned grid_of() { return (unsigned)(pitch_f / 256); }

void ref_pair(int kind, float4 *force, unsigned *nnlist, unsigned *nnlist_max)
{
    emu_launch(grid_of(), 256, [&] {
        if (kind == 0) pair_forces(force, nnlist, nnlist_max);
        else pair_forces_ewa(force, nnlist, nnlist_max);
    });
}
void ref_bonds(float4 *force, uint2 *bl, unsigned *blm) { emu_launch(grid_of(), 256, [&] { bonded_forces(force, bl, blm); }); }
void ref_angles(float4 *force, uint4 *al, unsigned *alm) { emu_launch(grid_of(), 256, [&] { angle_forces(force, al, alm); }); }
void ref_leapfrog_nve(float4 *pos, float4 *vel, float4 *force) { emu_launch(grid_of(), 256, [&] { leapfrog_nve(pos, vel, force); }); }
void ref_leapfrog_nvt(float4 *pos, float4 *vel, float4 *force, float scale, float *ke)
{
    emu_launch(grid_of(), 256, [&] { leapfrog_nvt_berendsen(pos, vel, force, scale, ke); });
}
void ref_ke_sum(float *ke) { emu_launch(1, nblocks, [&] { kinetic_energy_sum(ke); }); }
void ref_vv_pre(float4 *pos, float4 *vel, float4 *force) { emu_launch(grid_of(), 256, [&] { vverlet_nve_pre(pos, vel, force); }); }
void ref_vv_cor(float4 *vel, float4 *force) { emu_launch(grid_of(), 256, [&] { vverlet_nve_cor(vel, force); }); }
