// NESTA and SimpleMRIRecon through the OpenCLIPER-style C++ facade, in the
// shape of the reference driver tests/MRIRecon.cpp:94-235 (create the runtime,
// wrap the data, create the process, init, set launch parameters, launch).
// Reads raw little-endian inputs written by tests/test_facade_gpu.py:
//   <dir>/dims.u32 = W H F C, y.c64 [F][C][H][W], S.c64 [C][H][W], rowmask.u32 [F][H],
//   xn.f32 [2][F][H][W], xmesh.i32 [2][W][H], bb.u32 [4] (motion compensation)
// and writes x.c64 [F][H][W], simple.c64 [H][W] (frame 0 data), mc.c64 and
// mcadj.c64 (MotionCompensation / AdjointMotionCompensation of x), xmc.c64
// (NestaUp with argsMC started from x), stats.txt.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include <OpenCLIPER/CLapp.hpp>
#include <OpenCLIPER/KData.hpp>
#include <OpenCLIPER/XData.hpp>
#include <OpenCLIPER/processes/AdjointMotionCompensation.hpp>
#include <OpenCLIPER/processes/MotionCompensation.hpp>
#include <OpenCLIPER/processes/examples/SimpleMRIRecon.hpp>
#include <OpenCLIPER/processes/nesta/NestaUp.hpp>

using namespace OpenCLIPER;

template <typename T>
static std::vector<T> readRaw(const std::string& path, size_t n) {
  std::vector<T> v(n);
  std::ifstream f(path, std::ios::binary);
  f.read(reinterpret_cast<char*>(v.data()), std::streamsize(n * sizeof(T)));
  if (!f) throw std::runtime_error("cannot read " + path);
  return v;
}

template <typename T>
static void writeRaw(const std::string& path, const std::vector<T>& v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(v.data()), std::streamsize(v.size() * sizeof(T)));
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::cerr << "usage: " << argv[0] << " <dir>\n";
    return 2;
  }
  const std::string dir = argv[1];
  try {
    const auto dims = readRaw<uint32_t>(dir + "/dims.u32", 4);
    const dimIndexType W = dims[0], H = dims[1], F = dims[2], C = dims[3];
    auto pCLapp = CLapp::create();
    auto sens = std::make_shared<SensitivityMapsData>(pCLapp, W, H, C, readRaw<complexType>(dir + "/S.c64", size_t(W) * H * C));
    auto masks = SamplingMasksData::fromRowMask(pCLapp, W, H, F, readRaw<uint32_t>(dir + "/rowmask.u32", size_t(H) * F));
    auto pInputKData = std::make_shared<KData>(pCLapp, W, H, F, C,
                                               readRaw<complexType>(dir + "/y.c64", size_t(W) * H * F * C), sens, masks);
    auto nestaUpProcess = Process::create<NestaUp>(pCLapp);
    pCLapp->loadKernels();
    auto pOutputXData = std::make_shared<XData>(pCLapp, pInputKData);
    nestaUpProcess->setInput(pInputKData);
    nestaUpProcess->setOutput(pOutputXData);
    nestaUpProcess->init();
    // tests/MRIRecon.cpp:105-114 parameters, fewer iterations
    auto params = std::make_shared<NestaUp::LaunchParameters>(1e-2f, 3e-4f, 1.0f, 4u, 3e-4f, 1, 30, 1u, 7u, nullptr, false);
    nestaUpProcess->setLaunchParameters(params);
    nestaUpProcess->launch();
    std::vector<complexType> x;
    pOutputXData->device2Host(x);
    writeRaw(dir + "/x.c64", x);
    std::ofstream st(dir + "/stats.txt");
    const auto& s = nestaUpProcess->getStats();
    st << s.normU << " " << s.inner_iters << " " << params->tolVar << "\n";

    // SimpleMRIRecon on the same k-space (src/processes/examples/SimpleMRIRecon.cpp:80-101)
    auto simple = Process::create<SimpleMRIRecon>(pCLapp);
    auto pSimpleOut = std::make_shared<XData>(pCLapp, pInputKData);
    simple->setInput(pInputKData);
    simple->setOutput(pSimpleOut);
    simple->init();
    simple->launch();
    std::vector<complexType> xs;
    pSimpleOut->device2Host(xs);
    writeRaw(dir + "/simple.c64", xs);

    // motion compensation: the operators on x, then NestaUp with argsMC
    // started from x (the reference's motion-compensated pass reuses the
    // output XData of the first reconstruction)
    ArgumentsMotionCompensation args;
    args.xnData = std::make_shared<ArrayData<float>>(pCLapp, readRaw<float>(dir + "/xn.f32", 2 * size_t(F) * H * W));
    args.xData = std::make_shared<ArrayData<int>>(pCLapp, readRaw<int>(dir + "/xmesh.i32", 2 * size_t(W) * H));
    const auto bbv = readRaw<uint32_t>(dir + "/bb.u32", 4);
    std::vector<dimIndexType> bb(bbv.begin(), bbv.end());
    args.bound_box = &bb;
    auto mcOut = std::make_shared<XData>(pCLapp, pInputKData);
    auto mc = Process::create<MotionCompensation>(pCLapp);
    mc->setInput(pOutputXData);
    mc->setOutput(mcOut);
    mc->setLaunchParameters(std::make_shared<MotionCompensation::LaunchParameters>(&args));
    mc->init();
    mc->launch();
    std::vector<complexType> h;
    mcOut->device2Host(h);
    writeRaw(dir + "/mc.c64", h);
    auto adj = Process::create<AdjointMotionCompensation>(pCLapp);
    adj->setInput(pOutputXData);
    adj->setOutput(mcOut);
    adj->setLaunchParameters(std::make_shared<AdjointMotionCompensation::LaunchParameters>(&args));
    adj->init();
    adj->launch();
    mcOut->device2Host(h);
    writeRaw(dir + "/mcadj.c64", h);
    auto mcParams = std::make_shared<NestaUp::LaunchParameters>(1e-2f, 3e-4f, 1.0f, 1u, 3e-4f, 1, 20, 0u, 7u, &args);
    nestaUpProcess->setLaunchParameters(mcParams);
    nestaUpProcess->launch();
    pOutputXData->device2Host(h);
    writeRaw(dir + "/xmc.c64", h);
    st << s.normU << " " << s.inner_iters << " " << s.status << "\n";

    // the reference's error behaviour: a bounding box that is not 4 values is refused
    bb.push_back(1);
    try {
      nestaUpProcess->launch();
      std::cerr << "expected std::invalid_argument\n";
      return 3;
    } catch (const std::invalid_argument& e) {
      st << "refused bound_box\n";
    }
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
