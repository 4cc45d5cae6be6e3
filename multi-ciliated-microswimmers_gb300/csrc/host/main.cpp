// `cilia sim.cfg`: the drop-in driver (src/main.cpp:48-148).  Reads the cfg,
// builds the Simulation on the GPU engine, runs it to `desiredt`, writes the
// checkpoint files and the cfg back with the new `globalt`.
//
// Optional cfg keys beyond the reference's schema (defaults keep the
// reference's behaviour): ststep (MD step, 0.001), seed (generator seed),
// precision ("fp64" | "fp32"), walls ("none" | "noslip" | "slip"), gravity,
// bead_mass (5), device.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>

#include "libconfig_lite.hpp"
#include "objects.hpp"

namespace {

void save_seed(const char* path, unsigned long long seed) {
  std::ofstream out(path, std::ios::out | std::ios::app);
  out << seed << "\n";
}

int from_cfg_file(const std::string& filename) {
  libconfig::Config cfg;
  std::cout << "loading: " << filename << std::endl;
  try {
    cfg.readFile(filename.c_str());
  } catch (const libconfig::FileIOException&) {
    std::cerr << "I/O error while reading file." << std::endl;
    return 1;
  } catch (const libconfig::ParseException& pex) {
    std::cerr << "Parse error at " << pex.getFile() << ":" << pex.getLine() << " - " << pex.getError() << std::endl;
    return 1;
  }
  libconfig::Setting& root = cfg.getRoot();
  cilia::SimOptions opt;
  try {
    std::string s;
    if (root.lookupValue("precision", s)) opt.precision = s == "fp32" ? MPCD_FP32 : MPCD_FP64;
    if (root.lookupValue("walls", s)) opt.walls = s == "noslip" ? MPCD_WALLS_NOSLIP : s == "slip" ? MPCD_WALLS_SLIP : MPCD_WALLS_NONE;
    root.lookupValue("gravity", opt.gravity);
    root.lookupValue("bead_mass", opt.bead_mass);
    root.lookupValue("device", opt.device);
    std::string name = root["name"];
    std::cout << "Simulation " << name << std::endl << std::endl << " MD Objects:" << std::endl << std::endl;
    cilia::Simulation sim(root, opt);
    save_seed("inital_randi.dat", sim.seed);
    std::cout << "T=" << sim.wc.globalt << "->" << sim.wc.desiredt << std::endl;
    sim.debug("mpcd.san");
    sim.run();
    sim.sync_from_device();
    sim.save_all();
    sim.wc.saveparameter(root);
    cfg.writeFile(filename.c_str());
    save_seed("end_randi.dat", sim.seed);
  } catch (const libconfig::SettingNotFoundException& nfex) {
    std::cerr << "No " << nfex.getPath() << " setting in configuration file." << std::endl;
    return 1;
  } catch (const libconfig::SettingTypeException& ex) {
    std::cerr << "error with:" << ex.getPath() << std::endl;
    return 1;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 0;
}

}  // namespace

int main(int argc, char* argv[]) {
  if (argc != 2) {
    std::cerr << "usage " << argv[0] << " <configfile>" << std::endl;
    return 1;
  }
  return from_cfg_file(argv[1]);
}
