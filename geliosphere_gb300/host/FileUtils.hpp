// Output-directory handling with the reference's side effects
// (Utils/include/FileUtils.hpp:27-53, Utils/src/FileUtils.cpp:15-124): the
// simulation chdir()s into results/<model>/<destination>/ and writes its
// files there; simulation_log.txt records the run parameters.
#pragma once
#include <string>

class ParamsCarrier;

// mkdir (if needed) and chdir into `name`; 1 on success, -1 on failure.
int mkdirAndchdir(const std::string &name);
// results/<modelDirectory>/<destination>, created and entered.
bool createDirectory(const std::string &modelDirectory, const std::string &destination);
// Directory name from the current time and dt / K0 / V (FileUtils.cpp:76-97).
std::string getDirectoryName(ParamsCarrier *p);
// simulation_log.txt in the current directory (FileUtils.cpp:99-124).
void writeSimulationReportFile(ParamsCarrier *p);
