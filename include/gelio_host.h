/* gelio_host.h -- C ABI of the host drop-in layer (libgelio_host.so).
 *
 * The host layer is a C++ restatement of the reference application's host
 * side around the engine of gelio.h: argument parsing
 * (Input/src/ParseParams.cpp:16-178), settings (Input/src/TomlSettings.cpp:9-52),
 * the model algorithms and batch mode (Algorithm/src/GeliosphereAlgorithm.cpp
 * and its three siblings, Algorithm/src/BatchRun.cpp:26-365), the GPU model
 * entry points (CUDAKernel/src/GeliosphereGpuModel.cpp and siblings) and the spectrum writers
 * (Utils/src/ResultsUtils.cpp:16-131).  These functions expose it to C,
 * ctypes and tests; the `geliosphere` executable is gelio_host_main.
 */
#ifndef GELIO_HOST_H
#define GELIO_HOST_H

#include <stdint.h>

#include "gelio.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The application: parse argv, pick the algorithm by model name, run it.
 * Returns 0; -1 when parsing fails or the model is unknown; 1 when a
 * simulation or evaluation could not run on the GPU (no usable device, an
 * engine error), where the reference's gpuErrchk ends the process with the
 * CUDA error code (replaces main(), main.cpp:22-40). */
int32_t gelio_host_main(int32_t argc, char **argv);

/* Parse argv into the process-wide parameter map; 1 on success
 * (replaces ParseParams::parseParams, Input/src/ParseParams.cpp:16-178). */
int32_t gelio_host_parse(int32_t argc, char **argv);

/* Clear the process-wide parameter map (tests; no reference counterpart). */
void gelio_host_reset(void);

/* Typed reads of the parameter map with a default
 * (replace ParamsCarrier::getInt/getFloat/getString,
 * Input/include/ParamsCarrier.hpp:127-345).  get_string copies at most
 * cap-1 bytes and returns the full length. */
int32_t gelio_host_get_int(const char *key, int32_t dflt);
float gelio_host_get_float(const char *key, float dflt);
int32_t gelio_host_get_string(const char *key, const char *dflt, char *buf, int32_t cap);
/* ParamsCarrier::putInt/putFloat/putString (insert semantics for numbers). */
void gelio_host_put_int(const char *key, int32_t v);
void gelio_host_put_float(const char *key, float v);
void gelio_host_put_string(const char *key, const char *v);

/* Load a Settings.toml into the parameter map; 1 on success
 * (replaces TomlSettings::parseFromSettings, Input/src/TomlSettings.cpp:9-52). */
int32_t gelio_host_load_settings(const char *path);

/* gelio_sim_params the GPU model would run for `model` from the current
 * parameter map, with the precedence of setConstants
 * (CUDAKernel/src/CosmicConstants.cu:43-111). */
int32_t gelio_host_resolve(int32_t model, gelio_sim_params *out);

/* Resolve the rows of a batch CSV as batch mode does, without running them:
 * each row that would run gets its results directory and simulation_log.txt
 * (relative to the current directory) and its gelio_sim_params in out[k]
 * with its 1-based CSV row in rows[k] (either may be NULL); at most cap are
 * copied and *n receives how many rows resolve.  GELIO_OK, or
 * GELIO_ERR_INVALID_ARGUMENT when the file cannot be read or its names are
 * not unique (replaces the planning half of BatchRun::runAlgorithm,
 * Algorithm/src/BatchRun.cpp:26-100). */
int32_t gelio_host_batch_plan(const char *csv_path, gelio_sim_params *out, int32_t *rows, int32_t cap,
                              int32_t *n);

/* Write one model's spectrum files (the evaluators' names and formats) for
 * `s` into directory `dir` (NULL = current); 0 on success
 * (replaces the writeSpectrum calls of Algorithm/src/TwoDimensionBpResults.cpp:103-133,
 * OneDimensionBpResults.cpp:87-112 and OneDimensionFpResults.cpp:88-113). */
int32_t gelio_host_write_spectra(int32_t model, const gelio_spectra *s, int32_t csv, const char *dir);

/* One log.dat line of an exit record as the GPU models print it
 * (GeliosphereModel.cu:442, OneDimensionBpModel.cu:192, OneDimensionFpModel.cu:195);
 * returns the length, copies at most cap-1 bytes. */
int32_t gelio_host_log_line(int32_t model, const gelio_exit_record *r, float theta_injection, char *buf,
                            int32_t cap);

/* Carrington rotation number of the 15th of month/year as a table key
 * (replaces MeasureValuesTransformation::getCarringtonRotation,
 * Input/src/MeasureValuesTransformation.cpp:83-115). */
int32_t gelio_host_carrington_rotation(int32_t month, int32_t year);

#ifdef __cplusplus
}
#endif
#endif
