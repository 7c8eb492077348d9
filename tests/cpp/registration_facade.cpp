// GroupwiseRegistration through the OpenCLIPER-style C++ facade, in the shape
// of the reference driver's motion loop (tests/MRIRecon.cpp:204-282): create
// the process, init with InitParameters, launch with argsMC and TData, reuse
// argsMC->TData on the next motion iteration, warp with MotionCompensation.
// Reads <dir>/dims.u32 = N F radius nmax and x.c64 [F][N][N]; writes T1.f32,
// xn1.f32, xmesh.i32, bb.u32, H1.f32 (first launch), T2.f32, xn2.f32 (second
// launch, started from T1), mc.c64 (MotionCompensation of x with the second
// estimate), stats.txt.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include <OpenCLIPER/CLapp.hpp>
#include <OpenCLIPER/XData.hpp>
#include <OpenCLIPER/processes/GroupwiseRegistration.hpp>
#include <OpenCLIPER/processes/MotionCompensation.hpp>

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
    std::cerr << "usage: registration_facade <dir>\n";
    return 2;
  }
  const std::string dir = argv[1];
  try {
    const auto dims = readRaw<uint32_t>(dir + "/dims.u32", 4);
    const uint32_t N = dims[0], F = dims[1], radius = dims[2], nmax = dims[3];
    auto pCLapp = CLapp::create();
    auto x = readRaw<complexType>(dir + "/x.c64", size_t(F) * N * N);
    auto pX = std::make_shared<XData>(pCLapp, N, N, F, x);

    // tests/MRIRecon.cpp:121-129 parameters, a smaller step and iteration count
    int Dp[2] = {4, 4};
    std::vector<float> lambda = {0.f, 0.005f, 0.f, 0.5f};
    auto gw = Process::create<GroupwiseRegistration>(pCLapp);
    gw->setInput(pX);
    gw->setInitParameters(
        std::make_shared<GroupwiseRegistration::InitParameters>(0.05f, true, radius, 3u, Dp, nmax, 0.01f, 0.005f, lambda));
    gw->init();
    ArgumentsMotionCompensation* argsMC = new ArgumentsMotionCompensation();
    std::shared_ptr<Data> TData;
    std::ofstream st(dir + "/stats.txt");
    for (int i = 0; i < 2; ++i) {
      auto params = std::make_shared<GroupwiseRegistration::LaunchParameters>(argsMC, TData, i);
      gw->setLaunchParameters(params);
      gw->launch();
      TData = argsMC->TData;  // MRIRecon.cpp:255: the next motion iteration starts from this T
      std::vector<float> T, xn, H = gw->getMetric();
      std::static_pointer_cast<ArrayData<float>>(argsMC->TData)->device2Host(T);
      std::static_pointer_cast<ArrayData<float>>(argsMC->xnData)->device2Host(xn);
      writeRaw(dir + "/T" + std::to_string(i + 1) + ".f32", T);
      writeRaw(dir + "/xn" + std::to_string(i + 1) + ".f32", xn);
      writeRaw(dir + "/H" + std::to_string(i + 1) + ".f32", H);
      st << gw->getStats().iterations << " " << gw->getStats().status << " " << gw->getControlPoints() << "\n";
    }
    std::vector<int> xm;
    std::static_pointer_cast<ArrayData<int>>(argsMC->xData)->device2Host(xm);
    writeRaw(dir + "/xmesh.i32", xm);
    std::vector<uint32_t> bb(argsMC->bound_box->begin(), argsMC->bound_box->end());
    writeRaw(dir + "/bb.u32", bb);

    auto mcOut = std::make_shared<XData>(pCLapp, N, N, F, x);
    auto mc = Process::create<MotionCompensation>(pCLapp);
    mc->setInput(pX);
    mc->setOutput(mcOut);
    mc->setLaunchParameters(std::make_shared<MotionCompensation::LaunchParameters>(argsMC));
    mc->init();
    mc->launch();
    std::vector<complexType> h;
    mcOut->device2Host(h);
    writeRaw(dir + "/mc.c64", h);

    // the reference's error behaviour: a whole-box region of interest (radius 0) is refused
    auto bad = Process::create<GroupwiseRegistration>(pCLapp);
    bad->setInput(pX);
    bad->setInitParameters(
        std::make_shared<GroupwiseRegistration::InitParameters>(1.f, true, 0u, 3u, Dp, nmax, 0.01f, 0.005f, lambda));
    try {
      bad->init();
      st << "accepted\n";
    } catch (const std::invalid_argument&) {
      st << "refused\n";
    }
    delete argsMC;
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
