// TEST INFRASTRUCTURE: the reference's own 2D Geliosphere CUDA sources,
// compiled here as one translation unit into oracle/_ref/ref_geliosphere.cubin
// (oracle/Makefile target `ref_gpu`, include paths into the reference tree).
// Nothing of the reference is copied into this repository; oracle/ref_gpu.py
// loads the cubin through the CUDA driver API to time the reference kernels
// on this GPU and to bin their exits.
#include "CosmicConstants.cu"
#include "CosmicUtils.cu"
#include "GeliosphereModel.cu"
