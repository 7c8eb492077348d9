// The MAT-file forms of the OpenCLIPER-style facade, in the shape of the
// reference's examples/simpleMRIRecon.cpp:60-112 (KData from a .mat file,
// SimpleMRIRecon, XData::matlabSave) plus NestaUp on the same data.
// Usage: mat_facade <kdata.mat> <outprefix>; writes <outprefix>_simple.mat,
// <outprefix>_nesta.mat, <outprefix>_k.mat (KData::matlabSave) and
// <outprefix>_stats.txt ("reload <max abs difference>", "async <error class of
// a failed asynchronous load>").
#include <algorithm>
#include <cmath>
#include <fstream>
#include <iostream>

#include <OpenCLIPER/CLapp.hpp>
#include <OpenCLIPER/KData.hpp>
#include <OpenCLIPER/XData.hpp>
#include <OpenCLIPER/processes/examples/SimpleMRIRecon.hpp>
#include <OpenCLIPER/processes/nesta/NestaUp.hpp>

using namespace OpenCLIPER;

int main(int argc, char** argv) {
  if (argc != 3) {
    std::cerr << "usage: " << argv[0] << " <kdata.mat> <outprefix>\n";
    return 2;
  }
  const std::string in = argv[1], out = argv[2];
  try {
    auto pCLapp = CLapp::create();
    // asynchronous load joined before use, as tests/MRIRecon.cpp:150-179 does
    auto pInputKData = std::make_shared<KData>(pCLapp, in, true);
    pInputKData->waitLoadEnd();
    auto pOutputXData = std::make_shared<XData>(pCLapp, pInputKData);
    auto pProcess = Process::create<SimpleMRIRecon>(pCLapp);
    pProcess->setInput(pInputKData);
    pProcess->setOutput(pOutputXData);
    pProcess->init();
    pProcess->launch();
    pOutputXData->matlabSave(out + "_simple.mat");

    // the saved image read back through XData(app, fileName)
    auto reloaded = std::make_shared<XData>(pCLapp, out + "_simple.mat");
    std::vector<complexType> a, b;
    pOutputXData->device2Host(a);
    reloaded->device2Host(b);
    float diff = a.size() == b.size() ? 0.f : INFINITY;
    for (size_t i = 0; i < std::min(a.size(), b.size()); ++i) diff = std::max(diff, std::abs(a[i] - b[i]));

    auto nesta = Process::create<NestaUp>(pCLapp);
    auto pNestaOut = std::make_shared<XData>(pCLapp, pInputKData);
    nesta->setInput(pInputKData);
    nesta->setOutput(pNestaOut);
    nesta->init();
    nesta->setLaunchParameters(
        std::make_shared<NestaUp::LaunchParameters>(0.01f, 1e-3f, 1.0f, 1u, 3e-4f, 1, 20, 0u, 7u, nullptr));
    nesta->launch();
    pNestaOut->matlabSave(out + "_nesta.mat");
    pInputKData->matlabSave(out + "_k.mat");
    // a failed asynchronous load reports its error when joined
    std::string async_err = "none";
    try {
      auto missing = std::make_shared<KData>(pCLapp, out + "_missing.mat", true);
      missing->waitLoadEnd();
    } catch (const std::invalid_argument&) {
      async_err = "invalid_argument";
    }
    std::ofstream(out + "_stats.txt") << "reload " << diff << "\nasync " << async_err << "\n";
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
