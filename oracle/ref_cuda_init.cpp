/*
 * ORACLE — test infrastructure only.
 *
 * The device set-up the reference's main() performs before any CUDA work (main.cpp:566, init_device from
 * cut/cuda_common.cpp: cudaSetDevice and the device properties its launch configurations read), for the build of
 * its own CUDA path (oracle/Makefile refcuda).
 */
#include "cut/cuda_common.h"

extern "C" void ref_init_device(int dev) { init_device(dev); }
