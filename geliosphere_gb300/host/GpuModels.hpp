// The GPU models behind the reference's interface
// (CUDAKernel/include/AbstractGpuSimulation.hpp:23-32): each
// prepareAndRunSimulation(ParamsCarrier*) resolves the parameters, enters
// results/<model>/<destination>/ like the reference (createDirectory), runs
// the simulation and its spectrum binning on the GB300 in one call, writes
// log.dat only when the log is kept (remove_log_files_after_simulation = 0)
// and writes simulation_log.txt.  The spectra are handed to the model's
// Results class.
#pragma once
class ParamsCarrier;

class AbstractGpuSimulation {
 public:
  virtual ~AbstractGpuSimulation() = default;
  virtual void prepareAndRunSimulation(ParamsCarrier *singleTone) = 0;
};

class OneDimensionFpGpuModel : public AbstractGpuSimulation {
 public:
  void prepareAndRunSimulation(ParamsCarrier *singleTone) override;   // OneDimensionFpGpuModel.cpp:7-40
};
class OneDimensionBpGpuModel : public AbstractGpuSimulation {
 public:
  void prepareAndRunSimulation(ParamsCarrier *singleTone) override;   // OneDimensionBpGpuModel.cpp:7-43
};
class SolarPropLikeGpuModel : public AbstractGpuSimulation {
 public:
  void prepareAndRunSimulation(ParamsCarrier *singleTone) override;   // SolarPropLikeGpuModel.cpp:7-44
};
class GeliosphereGpuModel : public AbstractGpuSimulation {
 public:
  void prepareAndRunSimulation(ParamsCarrier *singleTone) override;   // GeliosphereGpuModel.cpp:7-44
};

// Shared implementation; returns false if the run could not be made.
bool runGpuModel(ParamsCarrier *p, int model);
