// MAT-file (level 5) reader/writer of include/OpenCLIPER/gbn_matfile.hpp,
// without a GPU.  Usage:
//   matfile_selftest dump <in.mat> <outdir>   every numeric variable as
//       <outdir>/<name>.txt ("cls complex d0 d1 ...") + <name>.re / <name>.im
//       (the class's raw little-endian elements, MATLAB order)
//   matfile_selftest copy <in.mat> <out.mat>  read, then write all variables
//   matfile_selftest inflate <in.z> <out.bin> zlib stream -> bytes
#include <OpenCLIPER/gbn_matfile.hpp>

#include <fstream>
#include <iostream>
#include <iterator>

using namespace OpenCLIPER;

int main(int argc, char** argv) {
  if (argc != 4) {
    std::cerr << "usage: " << argv[0] << " dump|copy|inflate <in> <out>\n";
    return 2;
  }
  const std::string mode = argv[1], in = argv[2], out = argv[3];
  try {
    if (mode == "inflate") {
      std::ifstream f(in, std::ios::binary);
      std::vector<uint8_t> z((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
      const auto b = matfile::zlib_inflate(z.data(), z.size());
      std::ofstream(out, std::ios::binary).write(reinterpret_cast<const char*>(b.data()), std::streamsize(b.size()));
      return 0;
    }
    const auto vars = matfile::read(in);
    if (mode == "dump") {
      for (const auto& kv : vars) {
        const auto& v = kv.second;
        std::ofstream t(out + "/" + v.name + ".txt");
        t << v.cls << " " << int(v.complex);
        for (auto d : v.dims) t << " " << d;
        t << "\n";
        std::ofstream(out + "/" + v.name + ".re", std::ios::binary)
            .write(reinterpret_cast<const char*>(v.re.data()), std::streamsize(v.re.size()));
        if (v.complex)
          std::ofstream(out + "/" + v.name + ".im", std::ios::binary)
              .write(reinterpret_cast<const char*>(v.im.data()), std::streamsize(v.im.size()));
      }
      return 0;
    }
    if (mode == "copy") {
      std::vector<matfile::Var> all;
      for (const auto& kv : vars) all.push_back(kv.second);
      matfile::write(out, all);
      return 0;
    }
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  std::cerr << "unknown mode " << mode << "\n";
  return 2;
}
