// Process-wide access to the GB300 engine for the host layer, and the
// hand-off of fused spectra from a GPU model to its Results class (the
// reference passes them through log.dat, GeliosphereModel.cu:418-445).
#pragma once
#include <string>

#include "gelio.h"

class ParamsCarrier;

namespace ghost {

// The context on device 0, created on first use; nullptr (with an error
// message) when no usable GPU exists -- there is no CPU fallback.
gelio_ctx *context();

struct FusedSpectra {
  bool valid = false;
  int model = -1;
  gelio_spectra spectra;
};
FusedSpectra &lastFused();

// Set when a simulation or an evaluation could not run on the GPU (no usable
// device, an engine error): the executable then exits non-zero, as the
// reference does when gpuErrchk ends the process (CudaErrorCheck.cuh:31-41).
bool &runFailed();

// gelio_sim_params for `model` from the parameter map, with the precedence
// of setConstants / setSolarPropConstants / setGeliosphereModelConstants
// (CUDAKernel/src/CosmicConstants.cu:43-111) and the __constant__ defaults
// (CosmicConstants.cu:14-41).  The particle count is the reference's:
// ceil(millions * 1e6 / 4096) chunks of 4,096 (GeliosphereModel.cu:421).
gelio_sim_params resolveSimParams(ParamsCarrier *p, int model);

// Reference log.dat line of one exit record (the GPU writers,
// GeliosphereModel.cu:442, OneDimensionBpModel.cu:192, OneDimensionFpModel.cu:195).
std::string logLine(int model, const gelio_exit_record &r, float thetaInjection);

int modelFromName(const std::string &name);   // -1 if unknown
const char *modelDirectory(int model);        // results/<this>/...

}  // namespace ghost
