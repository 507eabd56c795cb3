/*
 * ref_driver.cu -- a small main program around the reference's own host
 * entry points, built against the compat-patched copy of its sources in
 * baseline/_ref/src (reference_cuda.py).  It stands in for the reference's
 * athom.cu, whose main hands argv[1] to SimulationInit, which appends ".inp"
 * to that string in place (simulation.cu:59); here the name lives in a
 * buffer with room for it.
 *
 *   ref_md run <name>           SimulationInit and SimulationRun (the
 *                               reference's SimulationRun_CUDA loop,
 *                               runGPU.cu:43-115) in the current directory;
 *                               prints the wall time of SimulationRun.  Its
 *                               SimulationFinish is not called: it frees the
 *                               force field's type names (FFieldFinish) and
 *                               then reads them to write the .xyz output
 *                               (ConfigFinish, simulation.cu:137-141,
 *                               323-328), which crashes the process
 *   ref_md forces <name> <out>  the reference's set-up (gpu_properties_init,
 *                               config_init, forces_init, neighborlist_init:
 *                               runGPU.cu:52-60, which builds the list) and one
 *                               forces() call; writes natom, the list lengths
 *                               (nnlist_max), the float4 forces, the list
 *                               pitch, the longest length and the list
 *                               columns up to it (nnlist[i + pitch*k]) to <out>
 */
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "config.h"
#include "forces.h"
#include "gpu_properties.h"
#include "neighborlist.h"
#include "simulation.h"

int main(int argc, char **argv)
{
    if (argc < 3) {
        std::fprintf(stderr, "usage: ref_md run <name> | ref_md forces <name> <out>\n");
        return 2;
    }
    std::setvbuf(stdout, nullptr, _IONBF, 0);   /* every line reaches the caller, even on a crash */
    static char name[4096];
    std::snprintf(name, sizeof(name) - 16, "%s", argv[2]);
    simulation *sim = SimulationInit(name);
    if (std::strcmp(argv[1], "run") == 0) {
        auto t0 = std::chrono::steady_clock::now();
        SimulationRun(sim);
        auto t1 = std::chrono::steady_clock::now();
        std::printf("REF_RUN_SECONDS %.6f\n", std::chrono::duration<double>(t1 - t0).count());
        return 0;
    }
    if (std::strcmp(argv[1], "forces") == 0 && argc >= 4) {
        config *conf = sim->conf;
        gpu_struct *g_prop = gpu_properties_init(conf);
        gpu_config *g_conf = config_init(conf);
        gpu_ffield *g_fld = forces_init(sim->fld, sim->pars, conf, g_prop, g_conf);
        gpu_nlist *g_nlist = neighborlist_init(conf, g_prop, sim->pars, g_conf, sim->fld);
        forces(g_prop, g_nlist, g_conf, g_fld, sim->fld, conf, sim->pars);
        cudaDeviceSynchronize();
        checkCUDAError("forces");
        config_DeviceToHost(conf, g_conf, 2);
        std::vector<unsigned> nmax(conf->natom);
        cudaMemcpy(nmax.data(), g_nlist->nnlist_max, sizeof(unsigned) * conf->natom, cudaMemcpyDeviceToHost);
        checkCUDAError("copy");
        FILE *f = std::fopen(argv[3], "wb");
        if (!f) return 3;
        std::fwrite(&conf->natom, sizeof(int), 1, f);
        std::fwrite(nmax.data(), sizeof(unsigned), conf->natom, f);
        std::fwrite(conf->force, sizeof(float4), conf->natom, f);
        unsigned mx = 0;
        for (int i = 0; i < conf->natom; i++) mx = nmax[i] > mx ? nmax[i] : mx;
        const int pitch = g_prop->dimGrid.x * g_prop->dimBlock.x;
        std::vector<unsigned> rows((size_t)pitch * mx);
        if (mx > 0)
            cudaMemcpy(rows.data(), g_nlist->nnlist, sizeof(unsigned) * rows.size(), cudaMemcpyDeviceToHost);
        checkCUDAError("copy list");
        std::fwrite(&pitch, sizeof(int), 1, f);
        std::fwrite(&mx, sizeof(unsigned), 1, f);
        std::fwrite(rows.data(), sizeof(unsigned), rows.size(), f);
        std::fclose(f);
        return 0;
    }
    std::fprintf(stderr, "unknown mode %s\n", argv[1]);
    return 2;
}
