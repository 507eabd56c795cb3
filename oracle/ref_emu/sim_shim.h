/*
 * sim_shim.h -- prefix for compiling the reference's simulation.cu (the
 * .inp/.fld/.cfg parsers) with g++.  FFieldInput writes 64 floats into the
 * 8-float bnd1/bnd2/ang1/ang2 buffers (simulation.cu:219-238); allocations in
 * that file are padded so the run stays inside its own memory.
 * TEST INFRASTRUCTURE.
 */
#include "cuda_shim.h"
#include <string>
#include <iostream>
#include <fstream>
#include <time.h>
extern "C" void *ref_pad_malloc(size_t n);
#define malloc(n) ref_pad_malloc(n)
