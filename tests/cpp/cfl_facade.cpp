// File-based drop-in path through the C++ facade: KData(app, fileName) from the
// CFL form, SimpleMRIRecon, SimpleMRIReconSOS and NestaUp, results saved with
// XData::saveCFLData.  Usage: cfl_facade <kdata file> <output prefix>
#include <OpenCLIPER/CLapp.hpp>
#include <OpenCLIPER/KData.hpp>
#include <OpenCLIPER/XData.hpp>
#include <OpenCLIPER/processes/examples/SimpleMRIRecon.hpp>
#include <OpenCLIPER/processes/examples/SimpleMRIReconSOS.hpp>
#include <OpenCLIPER/processes/nesta/NestaUp.hpp>

#include <cstdio>

using namespace OpenCLIPER;

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  try {
    auto app = CLapp::create();
    auto k = std::make_shared<KData>(app, std::string(argv[1]), true);  // asynchronous: accessors join the load
    const std::string out = argv[2];

    auto simple = Process::create<SimpleMRIRecon>(app);
    auto xs = std::make_shared<XData>(app, k);
    simple->setInput(k);
    simple->setOutput(xs);
    simple->init();
    simple->launch();
    xs->saveCFLData(out + "_simple");

    auto sos = Process::create<SimpleMRIReconSOS>(app);
    auto xo = std::make_shared<XData>(app, k);
    sos->setInput(k);
    sos->setOutput(xo);
    sos->init();
    sos->launch();
    xo->saveCFLData(out + "_sos");

    auto nesta = Process::create<NestaUp>(app);
    auto xn = std::make_shared<XData>(app, k);
    nesta->setInput(k);
    nesta->setOutput(xn);
    nesta->init();
    nesta->setLaunchParameters(std::make_shared<NestaUp::LaunchParameters>(0.01f, 1e-3f, 1.0f, 1u, 3e-4f, 0, 20, 0u, 7u, nullptr));
    nesta->launch();
    xn->saveCFLData(out + "_nesta");
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
