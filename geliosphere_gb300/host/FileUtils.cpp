#include "FileUtils.hpp"

#include <cerrno>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <dirent.h>
#include <sys/stat.h>
#include <unistd.h>

#include "ParamsCarrier.hpp"

int mkdirAndchdir(const std::string &name) {
  DIR *dir = opendir(name.c_str());
  if (dir) {
    closedir(dir);
    if (chdir(name.c_str()) != 0) {
      std::printf("ERROR %d: unable to change directory; %s\n", errno, std::strerror(errno));
      return -1;
    }
    return 1;
  }
  if (errno != ENOENT) {
    std::printf("ERROR: unable to open directory");
    return -1;
  }
  if (mkdir(name.c_str(), S_IRWXU | S_IRWXG | S_IROTH | S_IXOTH) != 0) {
    std::printf("ERROR %d: unable to mkdir; %s\n", errno, std::strerror(errno));
    return -1;
  }
  if (chdir(name.c_str()) != 0) {
    std::printf("ERROR %d: unable to change directory; %s\n", errno, std::strerror(errno));
    return -1;
  }
  return 1;
}

bool createDirectory(const std::string &modelDirectory, const std::string &destination) {
  return mkdirAndchdir("results") == 1 && mkdirAndchdir(modelDirectory) == 1 && mkdirAndchdir(destination) == 1;
}

std::string getDirectoryName(ParamsCarrier *p) {
  time_t clk = time(nullptr);
  std::string d = ctime(&clk);
  if (!d.empty() && d.back() == '\n') d.pop_back();
  for (char &ch : d)
    if (ch == ' ') ch = '_';
  return d + "_dt=" + std::to_string(p->getFloat("dt", p->getFloat("dt_default", 50.0f))) + "K0=" +
         std::to_string(p->getFloat("K0", p->getFloat("K0_default", 0.000222f))) + "V=" +
         std::to_string(p->getFloat("V", p->getFloat("V_default", 2.66667e-6f)));
}

void writeSimulationReportFile(ParamsCarrier *p) {
  FILE *f = std::fopen("simulation_log.txt", "w");
  if (!f) return;
  const std::string model = p->getString("model", "1D Fp");
  std::fprintf(f, "Model: %s\n", model.c_str());
  std::fprintf(f, "---------------------\n");
  if (p->getInt("month_option", -1) != -1) {
    std::fprintf(f, "Selected month: %d\n", p->getInt("month_option", -1));
    std::fprintf(f, "Selected year: %d\n", p->getInt("year_option", -1));
  }
  if (model == "2D SolarProp-like") std::fprintf(f, "SolarProp-like model ratio: %g\n", p->getFloat("solarPropRatio", 0.02f));
  if (model == "2D Geliosphere") {
    std::fprintf(f, "Geliosphere model ratio: %g\n", p->getFloat("geliosphereRatio", 0.2f));
    std::fprintf(f, "C Delta: %g\n", p->getFloat("C_delta", 8.7e-5f));
    const float tilt = p->getFloat("tilt_angle", p->getFloat("default_tilt_angle", 0.1f));
    std::fprintf(f, "Loaded tilt angle from file: %g\n", tilt);
    std::fprintf(f, "Calculated tilt angle:: %g\n", tilt * 3.1415926535f / 180.0f);
  }
  std::fprintf(f, "dt: %g\n", p->getFloat("dt", p->getFloat("dt_default", 50.0f)));
  std::fprintf(f, "K0: %g\n", p->getFloat("K0", p->getFloat("K0_default", 0.000222f)));
  std::fprintf(f, "V: %g\n", p->getFloat("V", p->getFloat("V_default", 2.66667e-6f)));
  std::fclose(f);
}
