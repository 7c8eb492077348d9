// C++ facade with OpenCLIPER's Process-style API over the GB300 C ABI (gbn.h).
//
// Callers written against the reference (tests/MRIRecon.cpp,
// examples/simpleMRIRecon.cpp) keep their structure: create the runtime with
// CLapp::create, wrap k-space, sensitivity maps and sampling masks in
// KData/SensitivityMapsData/SamplingMasksData, create processes with
// Process::create<T>(app), set input/output and parameters, then init() and
// launch().  Differences from the reference:
//  - device buffers are CUDA allocations: Data::getDeviceBuffer() returning a
//    cl::Buffer* becomes Data::getDevicePtr() returning void*;
//  - data objects are built from host vectors (file loaders are not part of
//    this library);
//  - the motion-compensation meshes of ArgumentsMotionCompensation are
//    ArrayData<float> / ArrayData<int> built from host vectors (the reference
//    builds them inside GroupwiseRegistration, which is not part of this
//    library).
// Errors are thrown as CLError (code = GBN_ERR_*) or std::invalid_argument,
// like the reference's BTTHROW (LPISupport/include/LPISupport/Utils.hpp:67-83).
#pragma once

#include <complex>
#include <cstdint>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <exception>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../gbn.h"
#include "gbn_matfile.hpp"

namespace OpenCLIPER {

using dimIndexType = uint32_t;
using realType = float;
using complexType = std::complex<float>;

/// CLError (include/OpenCLIPER/CLapp.hpp:114-144): a runtime failure with a status code.
class CLError : public std::runtime_error {
 public:
  CLError(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int err() const { return code_; }

 private:
  int code_;
};

inline void gbnCheck(int rc, const char* where) {
  if (rc == GBN_OK) return;
  const std::string msg = std::string(where) + ": " + gbn_last_error_string();
  if (rc == GBN_ERR_INVALID) throw std::invalid_argument(msg);
  throw CLError(rc, msg);
}

/// CLapp (src/CLapp.cpp:188-575): device, stream and allocation layer.
class CLapp {
 public:
  struct PlatformTraits {};
  struct DeviceTraits {
    int device;
    DeviceTraits() : device(0) {}
    explicit DeviceTraits(int d) : device(d) {}
  };
  static std::shared_ptr<CLapp> create() { return create(PlatformTraits(), DeviceTraits()); }
  static std::shared_ptr<CLapp> create(const PlatformTraits&, const DeviceTraits& dt) {
    return std::shared_ptr<CLapp>(new CLapp(dt.device));
  }
  ~CLapp() {
    if (ctx_) gbn_ctx_destroy(ctx_);
  }
  CLapp(const CLapp&) = delete;
  CLapp& operator=(const CLapp&) = delete;
  gbn_ctx* ctx() const { return ctx_; }
  /// kernels are compiled ahead of time; kept for source compatibility
  void loadKernels() {}
  /// getCommandQueue().finish()
  void finish() { gbnCheck(gbn_ctx_sync(ctx_), "CLapp::finish"); }

 private:
  explicit CLapp(int device) { gbnCheck(gbn_ctx_create(device, &ctx_), "CLapp::create"); }
  gbn_ctx* ctx_ = nullptr;
};

/// Data (src/Data.cpp): one contiguous device buffer mirroring a host array.
class Data {
 public:
  virtual ~Data() {
    if (dev_ && app_) gbn_free(app_->ctx(), dev_);
  }
  Data(const Data&) = delete;
  Data& operator=(const Data&) = delete;
  void* getDevicePtr() const {
    ensureLoaded();
    return dev_;
  }
  size_t getBytes() const {
    ensureLoaded();
    return bytes_;
  }
  const std::shared_ptr<CLapp>& getApp() const { return app_; }
  /// Data::waitLoadEnd (Data.cpp:1110-1115): waits for an asynchronous file
  /// load to finish; a no-op for data that were loaded synchronously.
  void waitLoadEnd() const { ensureLoaded(); }

 protected:
  Data(const std::shared_ptr<CLapp>& app, size_t bytes) : app_(app), bytes_(bytes) {
    gbnCheck(gbn_alloc(app->ctx(), bytes, &dev_), "Data: device allocation");
  }
  // no device buffer yet (a load that completes later)
  explicit Data(const std::shared_ptr<CLapp>& app) : app_(app) {}
  void allocate(size_t bytes) {
    bytes_ = bytes;
    gbnCheck(gbn_alloc(app_->ctx(), bytes, &dev_), "Data: device allocation");
  }
  // completes a pending load (subclasses with asynchronous loads override it)
  virtual void ensureLoaded() const {}
  void upload(const void* host) {
    gbnCheck(gbn_upload(app_->ctx(), dev_, host, bytes_), "Data::host2Device");
    app_->finish();
  }
  void download(void* host) const { gbnCheck(gbn_download(app_->ctx(), host, dev_, bytes_), "Data::device2Host"); }
  std::shared_ptr<CLapp> app_;
  void* dev_ = nullptr;
  size_t bytes_ = 0;
};

namespace cfl {
// LPISupport::Utils::basename (LPISupport/src/Utils.cpp:123-132): the name
// without its last extension
inline std::string basename(const std::string& f) {
  const size_t p = f.find_last_of('.');
  return p == std::string::npos ? f : f.substr(0, p);
}
inline bool exists(const std::string& f) { return std::ifstream(f).good(); }
// reads exactly `count` elements of T from the start of a raw file
template <typename T>
std::vector<T> read_raw(const std::string& f, size_t count, const char* who) {
  std::ifstream in(f, std::ios::binary);
  if (!in) throw std::invalid_argument(std::string(who) + ": cannot open " + f);
  std::vector<T> v(count);
  in.read(reinterpret_cast<char*>(v.data()), std::streamsize(count * sizeof(T)));
  if (size_t(in.gcount()) != count * sizeof(T))
    throw std::invalid_argument(std::string(who) + ": " + f + " holds fewer than the expected " +
                                std::to_string(count) + " elements");
  return v;
}
}  // namespace cfl

/// SensitivityMapsData: coil maps [C][H][W].
class SensitivityMapsData : public Data {
 public:
  SensitivityMapsData(const std::shared_ptr<CLapp>& app, dimIndexType W, dimIndexType H, dimIndexType C,
                      const std::vector<complexType>& maps)
      : Data(app, sizeof(complexType) * size_t(W) * H * C), W_(W), H_(H), C_(C) {
    if (maps.size() != size_t(W) * H * C) throw std::invalid_argument("SensitivityMapsData: size mismatch");
    upload(maps.data());
  }
  dimIndexType getNCoils() const { return C_; }
  dimIndexType width() const { return W_; }
  dimIndexType height() const { return H_; }
  void device2Host(std::vector<complexType>& out) const {
    out.resize(size_t(W_) * H_ * C_);
    download(out.data());
  }

 private:
  dimIndexType W_, H_, C_;
};

/// SamplingMasksData: pixel mask [F][H][W], 0 = not sampled.  The row-mask
/// form (0/1 per phase-encode line, [F][H]) is expanded on the device like
/// SamplingMasksData::rowmask2pixelmask (SamplingMasksData.cpp:389-441).
class SamplingMasksData : public Data {
 public:
  SamplingMasksData(const std::shared_ptr<CLapp>& app, dimIndexType W, dimIndexType H, dimIndexType F,
                    const std::vector<uint8_t>& pixelMask)
      : Data(app, size_t(W) * H * F) {
    if (pixelMask.size() != size_t(W) * H * F) throw std::invalid_argument("SamplingMasksData: size mismatch");
    upload(pixelMask.data());
  }
  static std::shared_ptr<SamplingMasksData> fromRowMask(const std::shared_ptr<CLapp>& app, dimIndexType W,
                                                        dimIndexType H, dimIndexType F,
                                                        const std::vector<uint32_t>& rowMask) {
    if (rowMask.size() != size_t(H) * F) throw std::invalid_argument("SamplingMasksData: row mask size mismatch");
    auto m = std::shared_ptr<SamplingMasksData>(new SamplingMasksData(app, W, H, F));
    void* tmp = nullptr;
    gbnCheck(gbn_alloc(app->ctx(), rowMask.size() * 4, &tmp), "SamplingMasksData: row mask");
    int rc = gbn_upload(app->ctx(), tmp, rowMask.data(), rowMask.size() * 4);
    if (rc == GBN_OK)
      rc = gbn_op_rowmask_to_pixelmask(app->ctx(), static_cast<const uint32_t*>(tmp), static_cast<uint8_t*>(m->dev_),
                                       int(W), int(H), int(F));
    gbn_free(app->ctx(), tmp);
    gbnCheck(rc, "SamplingMasksData::rowmask2pixelmask");
    return m;
  }

 private:
  SamplingMasksData(const std::shared_ptr<CLapp>& app, dimIndexType W, dimIndexType H, dimIndexType F)
      : Data(app, size_t(W) * H * F) {}
};

namespace matio {
// The Dims variable (MatVarDimsData.cpp:41-67): uint32 [nSpatialDims,
// allSizesEqual, nCoils, nTemporalDims, temporal dims..., spatial dims...]
// with the spatial dims as (width, height).
struct Dims {
  dimIndexType W = 0, H = 0, C = 0, F = 1, nT = 0;
};
inline Dims parse_dims(const std::map<std::string, matfile::Var>& vars, const char* who) {
  const auto it = vars.find("Dims");
  if (it == vars.end()) throw std::invalid_argument("Error: no Dims variable in matlab file");
  const matfile::Var& v = it->second;
  if (v.complex || v.cls != matfile::kUInt32)
    throw std::invalid_argument("Matlab dims variable should be an array of 32 bits unsigned integers");
  const uint32_t* d = v.real<uint32_t>();
  const size_t n = v.numel();
  if (n < 4) throw std::invalid_argument(std::string(who) + ": Dims variable too short");
  const size_t nS = d[0], nT = d[3];
  if (n < 4 + nT + nS) throw std::invalid_argument(std::string(who) + ": Dims variable too short");
  if (nS != 2)
    throw std::invalid_argument(std::string(who) + ": only 2 spatial dimensions are supported (Dims says " +
                                std::to_string(nS) + ")");
  Dims r;
  r.C = d[2];
  r.nT = dimIndexType(nT);
  for (size_t i = 0; i < nT; ++i) r.F *= d[4 + i];
  r.W = d[4 + nT];
  r.H = d[5 + nT];
  return r;
}
inline matfile::Var dims_var(dimIndexType W, dimIndexType H, dimIndexType C, dimIndexType F) {
  const uint32_t d[7] = {2u, 1u, uint32_t(C), 1u, uint32_t(F), uint32_t(W), uint32_t(H)};
  matfile::Var v;
  v.name = "Dims";
  v.cls = matfile::kUInt32;
  v.dims = {1, 7};
  v.re.assign(reinterpret_cast<const uint8_t*>(d), reinterpret_cast<const uint8_t*>(d) + sizeof(d));
  return v;
}
// MATLAB (rows=H, cols=W, outer...) -> row-major complex [outer][H][W]
inline std::vector<complexType> complex_rows(const matfile::Var& v, const char* who) {
  if (v.cls != matfile::kSingle && v.cls != matfile::kDouble)
    throw std::invalid_argument(std::string(who) + ": Unsupported element data type in matlab data");
  std::vector<float> re, im;
  if (v.cls == matfile::kSingle) {
    matfile::to_row_major<float>(v, re, &im);
  } else {
    std::vector<double> r, i;
    matfile::to_row_major<double>(v, r, &i);
    re.assign(r.begin(), r.end());
    im.assign(i.begin(), i.end());
  }
  std::vector<complexType> out(re.size());
  for (size_t k = 0; k < re.size(); ++k) out[k] = complexType(re[k], im[k]);
  return out;
}
inline matfile::Var complex_var(const std::string& name, const std::vector<complexType>& rows, size_t H, size_t W,
                                const std::vector<uint64_t>& outer) {
  std::vector<float> re(rows.size()), im(rows.size());
  for (size_t k = 0; k < rows.size(); ++k) {
    re[k] = rows[k].real();
    im[k] = rows[k].imag();
  }
  return matfile::from_row_major<float>(name, matfile::kSingle, re.data(), im.data(), H, W, outer);
}
// MATLAB dims after (H, W) must equal `want`; trailing singleton dimensions may be absent
inline void check_dims(const matfile::Var& v, dimIndexType H, dimIndexType W, const std::vector<uint64_t>& want,
                       const char* who) {
  if (v.dims.size() < 2 || v.dims[0] != H || v.dims[1] != W)
    throw std::out_of_range(std::string("Invalid ") + who + " spatial dimensions");
  std::vector<uint64_t> got(v.dims.begin() + 2, v.dims.end()), w = want;
  while (!got.empty() && got.back() == 1) got.pop_back();
  while (!w.empty() && w.back() == 1) w.pop_back();
  if (got != w) throw std::out_of_range(std::string("Invalid ") + who + " dimensions");
}
}  // namespace matio

/// KData: multicoil k-space [F][C][H][W] with its sensitivity maps and masks.
class KData : public Data {
 public:
  KData(const std::shared_ptr<CLapp>& app, dimIndexType W, dimIndexType H, dimIndexType F, dimIndexType C,
        const std::vector<complexType>& data, std::shared_ptr<SensitivityMapsData> sens = nullptr,
        std::shared_ptr<SamplingMasksData> masks = nullptr)
      : Data(app, sizeof(complexType) * size_t(W) * H * F * C), W_(W), H_(H), F_(F), C_(C), sens_(sens), masks_(masks) {
    if (W % 8 != 0) throw std::invalid_argument("NDArray dimension 0 is not multiple of 8");
    if (data.size() != size_t(W) * H * F * C) throw std::invalid_argument("KData: size mismatch");
    upload(data.data());
  }
  /// KData(app, fileName, asyncLoad) (KData.cpp:276-435).  A MAT-file holds
  /// Dims, KData (single complex, MATLAB dims H x W [x C] x F) and, when
  /// present, SensitivityMaps (H x W x C) and SamplingMasks (uint32 row mask
  /// H x F, expanded to pixels, or uint8 pixel mask H x W x F).  Any other
  /// file is read in the CFL form (KData.cpp:246-351): header <base>.hdr
  /// (first line not starting with '#': "W H C F"), data `fileName` as raw
  /// complex float [F][C][H][W], sensitivity maps <base>_SensitivityMaps.cfl
  /// [C][H][W] and the sampling masks <base>_SamplingMasks.u32 (row mask
  /// [F][H]) or else <base>_SamplingMasks.u8 (pixel mask [F][H][W]), each
  /// when present.  Only 2-D Cartesian data.  With asyncLoad the files are
  /// read by a host thread (KData.cpp:281-284) while the caller goes on;
  /// waitLoadEnd() -- or any accessor -- joins it and moves the data to the
  /// device on the calling thread.  A read error is rethrown there.
  KData(const std::shared_ptr<CLapp>& app, const std::string& fileName, bool asyncLoad = false) : Data(app) {
    if (asyncLoad) {
      loader_.reset(new std::thread([this, fileName] {
        try {
          host_ = read_host(fileName);
        } catch (...) {
          error_ = std::current_exception();
        }
      }));
    } else {
      host_ = read_host(fileName);
      materialize();
    }
  }
  ~KData() override {
    if (loader_ && loader_->joinable()) loader_->join();  // as Data::~Data (Data.cpp:514)
  }
  std::shared_ptr<SensitivityMapsData> getSensitivityMapsData() const {
    ensureLoaded();
    return sens_;
  }
  std::shared_ptr<SamplingMasksData> getSamplingMasksData() const {
    ensureLoaded();
    return masks_;
  }
  dimIndexType getNCoils() const {
    ensureLoaded();
    return C_;
  }
  dimIndexType getDynDimsTotalSize() const {
    ensureLoaded();
    return F_;
  }
  dimIndexType width() const {
    ensureLoaded();
    return W_;
  }
  dimIndexType height() const {
    ensureLoaded();
    return H_;
  }
  void device2Host(std::vector<complexType>& out) const {
    ensureLoaded();
    out.resize(size_t(W_) * H_ * F_ * C_);
    download(out.data());
  }
  /// KData::matlabSave (KData.cpp:837-884): Dims, KData (H x W x C x F) and
  /// SensitivityMaps (H x W x C) when present; the sampling masks are not
  /// saved, as in the reference.  Written uncompressed.
  void matlabSave(const std::string& fileName) const {
    ensureLoaded();
    std::vector<matfile::Var> vars;
    vars.push_back(matio::dims_var(W_, H_, C_, F_));
    std::vector<complexType> h;
    device2Host(h);
    vars.push_back(matio::complex_var("KData", h, H_, W_, {C_, F_}));
    if (sens_) {
      sens_->device2Host(h);
      vars.push_back(matio::complex_var("SensitivityMaps", h, H_, W_, {C_}));
    }
    matfile::write(fileName, vars);
  }

 protected:
  void ensureLoaded() const override {
    if (!loader_) return;
    loader_->join();
    loader_.reset();
    if (error_) {
      std::exception_ptr e = error_;
      error_ = nullptr;
      std::rethrow_exception(e);
    }
    const_cast<KData*>(this)->materialize();
  }

 private:
  // a file's contents on the host
  struct HostK {
    dimIndexType W = 0, H = 0, F = 0, C = 0;
    std::vector<complexType> data, maps;
    std::vector<uint32_t> rowmask;
    std::vector<uint8_t> pixmask;
  };

  // the host data to the device (on the calling thread: a context is not shared across threads)
  void materialize() {
    HostK h = std::move(host_);
    if (h.W % 8 != 0) throw std::invalid_argument("NDArray dimension 0 is not multiple of 8");
    W_ = h.W;
    H_ = h.H;
    F_ = h.F;
    C_ = h.C;
    allocate(sizeof(complexType) * h.data.size());
    upload(h.data.data());
    if (!h.maps.empty()) sens_ = std::make_shared<SensitivityMapsData>(app_, h.W, h.H, h.C, h.maps);
    if (!h.rowmask.empty())
      masks_ = SamplingMasksData::fromRowMask(app_, h.W, h.H, h.F, h.rowmask);
    else if (!h.pixmask.empty())
      masks_ = std::make_shared<SamplingMasksData>(app_, h.W, h.H, h.F, h.pixmask);
  }

  static HostK read_mat(const std::string& fileName) {
    const auto vars = matfile::read(fileName);
    const matio::Dims d = matio::parse_dims(vars, "KData::KData");
    const auto it = vars.find("KData");
    if (it == vars.end()) throw std::invalid_argument("Error: no KData variable in matlab file");
    HostK h;
    h.W = d.W;
    h.H = d.H;
    h.F = d.F;
    h.C = d.C > 1 ? d.C : 1;
    matio::check_dims(it->second, h.H, h.W, {h.C, h.F}, "KData");
    h.data = matio::complex_rows(it->second, "KData");
    const auto sm = vars.find("SensitivityMaps");
    if (sm != vars.end()) {
      matio::check_dims(sm->second, h.H, h.W, {h.C}, "SensitivityMaps");
      h.maps = matio::complex_rows(sm->second, "SensitivityMaps");
    }
    const auto mk = vars.find("SamplingMasks");
    if (mk != vars.end()) {
      const matfile::Var& m = mk->second;
      if (m.complex) throw std::invalid_argument("Invalid mask format (supported: ROWMASK and PIXELMASK");
      if (m.cls == matfile::kUInt32) {  // row mask: MATLAB dims H x F (one 1-D array per frame)
        if (m.dims[0] != h.H || m.numel() != size_t(h.H) * h.F)
          throw std::out_of_range("Invalid SamplingMasks dimensions");
        const uint32_t* r = m.real<uint32_t>();
        h.rowmask.assign(r, r + m.numel());
      } else if (m.cls == matfile::kUInt8) {  // pixel mask: H x W x F
        matio::check_dims(m, h.H, h.W, {h.F}, "SamplingMasks");
        matfile::to_row_major<uint8_t>(m, h.pixmask, nullptr);
      } else {
        throw std::invalid_argument("Invalid mask format (supported: ROWMASK and PIXELMASK");
      }
    }
    return h;
  }

  static HostK read_host(const std::string& fileName) {
    if (matfile::is_mat(fileName)) return read_mat(fileName);
    const std::string base = cfl::basename(fileName);
    std::ifstream hdr(base + ".hdr");
    if (!hdr) throw std::invalid_argument("KData: cannot open " + base + ".hdr");
    HostK h;
    std::string line;
    bool ok = false;
    while (std::getline(hdr, line)) {
      if (line.empty() || line[0] == '#') continue;
      std::istringstream iss(line);
      if (!(iss >> h.W >> h.H >> h.C >> h.F))
        throw std::invalid_argument("Invalid line format: " + line + " (should be <width> <depth> <numCoils> <numFrames>)");
      ok = true;
      break;
    }
    if (!ok) throw std::invalid_argument("KData: no dimensions in " + base + ".hdr");
    h.data = cfl::read_raw<complexType>(fileName, size_t(h.W) * h.H * h.F * h.C, "KData");
    const std::string sname = base + "_SensitivityMaps.cfl";
    if (cfl::exists(sname)) h.maps = cfl::read_raw<complexType>(sname, size_t(h.W) * h.H * h.C, "SensitivityMapsData");
    const std::string rname = base + "_SamplingMasks.u32", pname = base + "_SamplingMasks.u8";
    if (cfl::exists(rname))
      h.rowmask = cfl::read_raw<uint32_t>(rname, size_t(h.H) * h.F, "SamplingMasksData");
    else if (cfl::exists(pname))
      h.pixmask = cfl::read_raw<uint8_t>(pname, size_t(h.W) * h.H * h.F, "SamplingMasksData");
    return h;
  }

  dimIndexType W_ = 0, H_ = 0, F_ = 0, C_ = 0;
  std::shared_ptr<SensitivityMapsData> sens_;
  std::shared_ptr<SamplingMasksData> masks_;
  HostK host_;
  mutable std::unique_ptr<std::thread> loader_;
  mutable std::exception_ptr error_;
};

/// XData: image series [F][H][W]; XData(app, kdata) sizes it like the input
/// k-space (XData.cpp:425-440).
class XData : public Data {
 public:
  XData(const std::shared_ptr<CLapp>& app, const std::shared_ptr<KData>& k)
      : Data(app, sizeof(complexType) * size_t(k->width()) * k->height() * k->getDynDimsTotalSize()),
        W_(k->width()), H_(k->height()), F_(k->getDynDimsTotalSize()) {}
  XData(const std::shared_ptr<CLapp>& app, dimIndexType W, dimIndexType H, dimIndexType F,
        const std::vector<complexType>& data)
      : Data(app, sizeof(complexType) * size_t(W) * H * F), W_(W), H_(H), F_(F) {
    if (W % 8 != 0) throw std::invalid_argument("NDArray dimension 0 is not multiple of 8");
    if (data.size() != size_t(W) * H * F) throw std::invalid_argument("XData: size mismatch");
    upload(data.data());
  }
  /// XData(app, fileName) from a MAT-file (XData.cpp:504-558): Dims and XData
  /// (single, MATLAB dims H x W x F; a real array gets a zero imaginary part).
  /// Image files (OpenCV) are not supported.
  XData(const std::shared_ptr<CLapp>& app, const std::string& fileName) : XData(load_mat(app, fileName)) {}
  dimIndexType getDynDimsTotalSize() const { return F_; }
  dimIndexType width() const { return W_; }
  dimIndexType height() const { return H_; }
  void device2Host(std::vector<complexType>& out) const {
    out.resize(size_t(W_) * H_ * F_);
    download(out.data());
  }
  /// XData::matlabSave (XData.cpp:886-930): Dims [2, 1, 0, 1, F, W, H] and
  /// XData (single complex, H x W x F).  Written uncompressed.
  void matlabSave(const std::string& fileName) const {
    std::vector<complexType> h;
    device2Host(h);
    matfile::write(fileName, {matio::dims_var(W_, H_, 0, F_), matio::complex_var("XData", h, H_, W_, {F_})});
  }
  /// XData::saveCFLData (XData.cpp:851-881): `fileName`.cfl raw complex float
  /// [F][H][W] and <basename(fileName)>.hdr "W H 1 F 1"; synchronous.
  void saveCFLData(const std::string& fileName, bool asyncSave = false) const {
    (void)asyncSave;
    std::vector<complexType> h;
    device2Host(h);
    std::ofstream out(fileName + ".cfl", std::ios::binary | std::ios::trunc);
    if (!out) throw std::invalid_argument("XData::saveCFLData: cannot write " + fileName + ".cfl");
    out.write(reinterpret_cast<const char*>(h.data()), std::streamsize(h.size() * sizeof(complexType)));
    std::ofstream hdr(cfl::basename(fileName) + ".hdr", std::ios::trunc);
    if (!hdr) throw std::invalid_argument("XData::saveCFLHeader: cannot write header");
    hdr << W_ << " " << H_ << " " << "1 " << F_ << " " << "1" << std::endl;
  }

 private:
  struct Loaded {
    std::shared_ptr<CLapp> app;
    dimIndexType W, H, F;
    std::vector<complexType> data;
  };
  explicit XData(Loaded&& l) : XData(l.app, l.W, l.H, l.F, l.data) {}
  static Loaded load_mat(const std::shared_ptr<CLapp>& app, const std::string& fileName) {
    if (!matfile::is_mat(fileName))
      throw std::invalid_argument("XData: " + fileName + " is not a MAT-file (image files are not supported)");
    const auto vars = matfile::read(fileName);
    const matio::Dims d = matio::parse_dims(vars, "XData::XData");
    const auto it = vars.find("XData");
    if (it == vars.end()) throw std::invalid_argument("Error: no XData variable in matlab file");
    if (d.C > 1) throw std::out_of_range("Invalid XData dimensions (XData has no coil dimension)");
    matio::check_dims(it->second, d.H, d.W, {d.F}, "XData");
    return Loaded{app, d.W, d.H, d.F, matio::complex_rows(it->second, "XData")};
  }
  dimIndexType W_, H_, F_;
};

/// Process / ProcessCore (include/OpenCLIPER/Process.hpp:49-108,
/// ProcessCore.hpp:56-270).
class Process {
 public:
  struct InitParameters {
    virtual ~InitParameters() {}
  };
  struct LaunchParameters {
    virtual ~LaunchParameters() {}
  };
  struct ProfileParameters {
    bool enable = false;
    unsigned long loops = 1;
    ProfileParameters() {}
    ProfileParameters(bool e, unsigned long l) : enable(e), loops(l) {}
    virtual ~ProfileParameters() {}
  };
  virtual ~Process() {}
  template <typename T>
  static std::shared_ptr<T> create(const std::shared_ptr<CLapp>& app,
                                   const std::shared_ptr<ProfileParameters>& pp = nullptr) {
    static_assert(std::is_base_of<Process, T>::value, "Process::create: class does not derive from Process");
    auto p = std::shared_ptr<T>(new T());
    p->app_ = app;
    p->pp_ = pp;
    return p;
  }
  void setInput(std::shared_ptr<Data> in) { in_ = std::move(in); }
  void setOutput(std::shared_ptr<Data> out) { out_ = std::move(out); }
  virtual void setInitParameters(const std::shared_ptr<InitParameters>& p) { ip_ = p; }
  virtual void setLaunchParameters(const std::shared_ptr<LaunchParameters>& p) { lp_ = p; }
  virtual void init() {
    if (!app_) throw std::invalid_argument("Invalid CLapp pointer");
  }
  virtual void launch() = 0;

 protected:
  Process() {}
  gbn_ctx* ctx() const { return app_->ctx(); }
  template <typename D>
  std::shared_ptr<D> inputAs(const char* who) const {
    auto d = std::dynamic_pointer_cast<D>(in_);
    if (!d) throw std::invalid_argument(std::string(who) + ": input data has the wrong type");
    return d;
  }
  template <typename D>
  std::shared_ptr<D> outputAs(const char* who) const {
    auto d = std::dynamic_pointer_cast<D>(out_);
    if (!d) throw std::invalid_argument(std::string(who) + ": output data has the wrong type");
    return d;
  }
  std::shared_ptr<CLapp> app_;
  std::shared_ptr<ProfileParameters> pp_;
  std::shared_ptr<Data> in_, out_;
  std::shared_ptr<InitParameters> ip_;
  std::shared_ptr<LaunchParameters> lp_;
};

/// TemporalTV (src/processes/nesta/TemporalTV.cpp:49-86) on XData.
class TemporalTV : public Process {
 public:
  enum Direction { FORWARD = 1, ADJOINT = 0 };
  struct InitParameters : Process::InitParameters {
    Direction dir;
    InitParameters(Direction d) : dir(d) {}
  };
  void launch() override {
    auto ip = std::dynamic_pointer_cast<InitParameters>(ip_);
    if (!ip) throw std::invalid_argument("TemporalTV: missing InitParameters");
    auto x = inputAs<XData>("TemporalTV");
    auto y = outputAs<XData>("TemporalTV");
    gbnCheck(gbn_op_ttv(ctx(), int(ip->dir), static_cast<const float*>(x->getDevicePtr()),
                        static_cast<float*>(y->getDevicePtr()), int(x->width()), int(x->height()),
                        int(x->getDynDimsTotalSize())),
             "TemporalTV::launch");
  }
};

/// VectorNormalization (src/processes/nesta/VectorNormalization.cpp:56-87).
class VectorNormalization : public Process {
 public:
  struct LaunchParameters : Process::LaunchParameters {
    float mu;
    LaunchParameters(float m) : mu(m) {}
  };
  void launch() override {
    auto lp = std::dynamic_pointer_cast<LaunchParameters>(lp_);
    if (!lp) throw std::invalid_argument("VectorNormalization: missing LaunchParameters");
    gbnCheck(gbn_op_normalize(ctx(), static_cast<const float*>(in_->getDevicePtr()), static_cast<float*>(out_->getDevicePtr()),
                              in_->getBytes() / sizeof(complexType), lp->mu),
             "VectorNormalization::launch");
  }
};

/// FFT process, 2-D over each image (src/processes/FFT.cpp:59-542).
class FFT : public Process {
 public:
  enum Direction { FORWARD = GBN_FFT_FORWARD, BACKWARD = GBN_FFT_BACKWARD };
  struct InitParameters : Process::InitParameters {
    int dim;
    std::shared_ptr<SamplingMasksData> samplingMask;
    explicit InitParameters(int d = -1, std::shared_ptr<SamplingMasksData> s = nullptr) : dim(d), samplingMask(s) {}
  };
  struct LaunchParameters : Process::LaunchParameters {
    Direction dir;
    explicit LaunchParameters(Direction d = FORWARD) : dir(d) {}
  };
  void init() override {
    Process::init();
    auto ip = std::dynamic_pointer_cast<InitParameters>(ip_);
    if (ip && (ip->dim != -1 || ip->samplingMask))
      throw CLError(GBN_ERR_UNSUPPORTED, "FFT::init: only full 2-D transforms (dim = -1) are implemented");
  }
  void launch() override {
    auto lp = std::dynamic_pointer_cast<LaunchParameters>(lp_);
    const Direction d = lp ? lp->dir : FORWARD;
    int W, H, batch;
    if (auto k = std::dynamic_pointer_cast<KData>(in_)) {
      W = int(k->width()), H = int(k->height()), batch = int(k->getDynDimsTotalSize() * k->getNCoils());
    } else {
      auto x = inputAs<XData>("FFT");
      W = int(x->width()), H = int(x->height()), batch = int(x->getDynDimsTotalSize());
    }
    if (in_->getBytes() != out_->getBytes())
      throw CLError(GBN_ERR_INVALID, "FFT: inputData and outputData must have the same number of images");
    gbnCheck(gbn_op_fft2(ctx(), int(d), static_cast<const float*>(in_->getDevicePtr()),
                         static_cast<float*>(out_->getDevicePtr()), W, H, batch),
             "FFT::launch");
  }
};

/// ComplexElementProd (src/processes/ComplexElementProd.cpp:64-131).
class ComplexElementProd : public Process {
 public:
  enum ConjugateSensMap_t { notConjugate = 0, conjugate = 1 };
  struct LaunchParameters : Process::LaunchParameters {
    ConjugateSensMap_t conjugateSensMap;
    std::shared_ptr<SensitivityMapsData> sensitivityMapsData;
    LaunchParameters(ConjugateSensMap_t c, const std::shared_ptr<SensitivityMapsData>& m)
        : conjugateSensMap(c), sensitivityMapsData(m) {}
  };
  void launch() override {
    auto lp = std::dynamic_pointer_cast<LaunchParameters>(lp_);
    if (!lp || !lp->sensitivityMapsData)
      throw std::invalid_argument("ComplexElementProd::launch: non-existing SensitivityMaps");
    auto out = outputAs<KData>("ComplexElementProd");
    const bool inK = bool(std::dynamic_pointer_cast<KData>(in_));
    gbnCheck(gbn_op_sensmul(ctx(), int(lp->conjugateSensMap), static_cast<const float*>(in_->getDevicePtr()), inK ? 1 : 0,
                            static_cast<const float*>(lp->sensitivityMapsData->getDevicePtr()),
                            static_cast<float*>(out->getDevicePtr()), int(out->width()), int(out->height()),
                            int(out->getDynDimsTotalSize()), int(out->getNCoils())),
             "ComplexElementProd::launch");
  }
};

/// XImageSum (src/processes/XImageSum.cpp:79-96): coil sum.
class XImageSum : public Process {
 public:
  void launch() override {
    auto k = inputAs<KData>("XImageSum");
    gbnCheck(gbn_op_coilsum(ctx(), static_cast<const float*>(k->getDevicePtr()), static_cast<float*>(out_->getDevicePtr()),
                            int(k->width()), int(k->height()), int(k->getDynDimsTotalSize()), int(k->getNCoils())),
             "XImageSum::launch");
  }
};

/// ApplyMask (src/processes/ApplyMask.cpp:21-51), in place on the input KData.
class ApplyMask : public Process {
 public:
  struct LaunchParameters : Process::LaunchParameters {
    std::shared_ptr<SamplingMasksData> samplingMasksData;
    explicit LaunchParameters(const std::shared_ptr<SamplingMasksData>& m) : samplingMasksData(m) {}
  };
  void launch() override {
    auto lp = std::dynamic_pointer_cast<LaunchParameters>(lp_);
    if (!lp || !lp->samplingMasksData) throw std::invalid_argument("Empty sampling masks data");
    auto k = inputAs<KData>("ApplyMask");
    gbnCheck(gbn_op_mask(ctx(), static_cast<float*>(k->getDevicePtr()),
                         static_cast<const uint8_t*>(lp->samplingMasksData->getDevicePtr()), int(k->width()),
                         int(k->height()), int(k->getDynDimsTotalSize()), int(k->getNCoils())),
             "ApplyMask::launch");
  }
};

/// ComplexAbs / ComplexAbsPow2 (complexAbs.cl:43-70, complexAbsPow2.cl:43-71).
class ComplexAbs : public Process {
 public:
  void launch() override {
    gbnCheck(gbn_op_abs(ctx(), static_cast<const float*>(in_->getDevicePtr()), static_cast<float*>(out_->getDevicePtr()),
                        in_->getBytes() / sizeof(complexType)),
             "ComplexAbs::launch");
  }
};
class ComplexAbsPow2 : public Process {
 public:
  void launch() override {
    gbnCheck(gbn_op_abs2(ctx(), static_cast<const float*>(in_->getDevicePtr()), static_cast<float*>(out_->getDevicePtr()),
                         in_->getBytes() / sizeof(complexType)),
             "ComplexAbsPow2::launch");
  }
};

/// SimpleMRIRecon (src/processes/examples/SimpleMRIRecon.cpp:58-101).
class SimpleMRIRecon : public Process {
 public:
  void launch() override {
    auto k = inputAs<KData>("SimpleMRIRecon");
    if (!k->getSensitivityMapsData()) throw std::invalid_argument("SimpleMRIRecon: missing sensitivity maps");
    gbnCheck(gbn_simple_recon(ctx(), static_cast<const float*>(k->getDevicePtr()),
                              static_cast<const float*>(k->getSensitivityMapsData()->getDevicePtr()),
                              static_cast<float*>(out_->getDevicePtr()), int(k->width()), int(k->height()),
                              int(k->getDynDimsTotalSize()), int(k->getNCoils())),
             "SimpleMRIRecon::launch");
  }
};

/// RSoS (src/processes/RSoS.cpp:43-85): root sum of squares over the coils of a
/// KData input into an XData output.
class RSoS : public Process {
 public:
  void launch() override {
    auto k = inputAs<KData>("RSoS");
    gbnCheck(gbn_op_rss(ctx(), static_cast<const float*>(k->getDevicePtr()), static_cast<float*>(out_->getDevicePtr()),
                        int(k->width()), int(k->height()), int(k->getDynDimsTotalSize()), int(k->getNCoils())),
             "RSoS::launch");
  }
};

/// SimpleMRIReconSOS (src/processes/examples/SimpleMRIReconSOS.cpp:54-118):
/// inverse FFT of every coil image, then RSoS.  The input KData is left as it
/// was (the reference transforms it in place and writes .mat / timing files).
class SimpleMRIReconSOS : public Process {
 public:
  void launch() override {
    auto k = inputAs<KData>("SimpleMRIReconSOS");
    gbnCheck(gbn_simple_recon_sos(ctx(), static_cast<const float*>(k->getDevicePtr()),
                                  static_cast<float*>(out_->getDevicePtr()), int(k->width()), int(k->height()),
                                  int(k->getDynDimsTotalSize()), int(k->getNCoils())),
             "SimpleMRIReconSOS::launch");
  }
};

/// A typed device array built from a host vector: the meshes of
/// ArgumentsMotionCompensation.
template <typename T>
class ArrayData : public Data {
 public:
  ArrayData(const std::shared_ptr<CLapp>& app, const std::vector<T>& host)
      : Data(app, sizeof(T) * host.size()), n_(host.size()) {
    if (host.empty()) throw std::invalid_argument("ArrayData: empty array");
    upload(host.data());
  }
  /// n elements on the device, contents undefined (filled by a process)
  ArrayData(const std::shared_ptr<CLapp>& app, size_t n) : Data(app, sizeof(T) * n), n_(n) {
    if (n == 0) throw std::invalid_argument("ArrayData: empty array");
  }
  size_t size() const { return n_; }
  void device2Host(std::vector<T>& host) const {
    host.resize(n_);
    download(host.data());
  }

 private:
  size_t n_;
};

/// ArgumentsMotionCompensation (include/OpenCLIPER/processes/
/// GroupwiseRegistration.hpp:95-100): xnData = deformed mesh [2][F][H][W]
/// float, xData = original mesh [2][W][H] int, both 1-based; bound_box = the
/// four 1-based bounding-box coordinates.  TData (the registration's B-spline
/// coefficients) is not read by the motion-compensation operators.
struct ArgumentsMotionCompensation {
  std::shared_ptr<Data> xnData;
  std::shared_ptr<Data> TData;
  std::shared_ptr<Data> xData;
  std::vector<dimIndexType>* bound_box;
};

namespace detail {
struct MotionArgs {
  const float* xn;
  const int* xmesh;
  int bb[4];
};
inline MotionArgs motion_args(const ArgumentsMotionCompensation* a, dimIndexType W, dimIndexType H,
                              dimIndexType F, const char* who) {
  if (!a || !a->xnData || !a->xData || !a->bound_box)
    throw std::invalid_argument(std::string(who) + ": ArgumentsMotionCompensation needs xnData, xData and bound_box");
  if (a->bound_box->size() != 4) throw std::invalid_argument(std::string(who) + ": bound_box must hold 4 values");
  if (a->xnData->getBytes() != sizeof(float) * 2 * size_t(F) * H * W)
    throw std::invalid_argument(std::string(who) + ": xnData must be float [2][F][H][W]");
  if (a->xData->getBytes() != sizeof(int) * 2 * size_t(W) * H)
    throw std::invalid_argument(std::string(who) + ": xData must be int [2][W][H]");
  MotionArgs m{static_cast<const float*>(a->xnData->getDevicePtr()), static_cast<const int*>(a->xData->getDevicePtr()),
               {0, 0, 0, 0}};
  for (int i = 0; i < 4; ++i) m.bb[i] = int((*a->bound_box)[size_t(i)]);
  return m;
}
}  // namespace detail

/// MotionCompensation (src/processes/MotionCompensation.cpp:57-78) and
/// AdjointMotionCompensation (src/processes/AdjointMotionCompensation.cpp:
/// 59-86): XData -> XData through the registration's meshes.
template <int Direction>
class MotionCompensationProcess : public Process {
 public:
  struct LaunchParameters : Process::LaunchParameters {
    ArgumentsMotionCompensation* argsMC;
    explicit LaunchParameters(ArgumentsMotionCompensation* args) : argsMC(args) {}
  };
  void launch() override {
    const char* who = Direction == GBN_TTV_FORWARD ? "MotionCompensation::launch" : "AdjointMotionCompensation::launch";
    auto lp = std::dynamic_pointer_cast<LaunchParameters>(lp_);
    if (!lp) throw std::invalid_argument(std::string(who) + ": missing LaunchParameters");
    auto in = inputAs<XData>(who);
    auto out = outputAs<XData>(who);
    if (in->width() != out->width() || in->height() != out->height() ||
        in->getDynDimsTotalSize() != out->getDynDimsTotalSize())
      throw std::invalid_argument(std::string(who) + ": input and output sizes differ");
    const auto m = detail::motion_args(lp->argsMC, in->width(), in->height(), in->getDynDimsTotalSize(), who);
    gbnCheck(gbn_op_motion(ctx(), Direction, static_cast<const float*>(in->getDevicePtr()),
                           static_cast<float*>(out->getDevicePtr()), m.xn, m.xmesh, m.bb, int(in->width()),
                           int(in->height()), int(in->getDynDimsTotalSize())),
             who);
  }
};
using MotionCompensation = MotionCompensationProcess<GBN_TTV_FORWARD>;
using AdjointMotionCompensation = MotionCompensationProcess<GBN_TTV_ADJOINT>;

/// GroupwiseRegistration (src/processes/GroupwiseRegistration.cpp:79-618,
/// groupwiseRegistration/optimizer.cpp; parameters GroupwiseRegistration.hpp:
/// 145-168): estimates the frames' motion of an XData [F][N][N] and fills
/// ArgumentsMotionCompensation for MotionCompensation and NestaUp.  As in the
/// reference, LaunchParameters::TData (the previous motion iteration's
/// argsMC->TData) starts the descent when given.  Errors are thrown as
/// std::invalid_argument (bad parameters, unsupported geometry) or CLError.
class GroupwiseRegistration : public Process {
 public:
  struct InitParameters : Process::InitParameters {
    float W;
    bool flagW;
    unsigned int radius;
    unsigned int E;
    int* Dp;
    unsigned int nmax;
    float et;
    float eh;
    std::vector<float> lambda;
    InitParameters(float W, bool flagW, unsigned int radius, unsigned int E, int* Dp, unsigned int nmax, float et,
                   float eh, const std::vector<float>& lambda)
        : W(W), flagW(flagW), radius(radius), E(E), Dp(Dp), nmax(nmax), et(et), eh(eh), lambda(lambda) {}
  };
  struct LaunchParameters : Process::LaunchParameters {
    ArgumentsMotionCompensation* argsMC;
    std::shared_ptr<Data> TData;
    int currentMotionIter;
    LaunchParameters(ArgumentsMotionCompensation* args, const std::shared_ptr<Data>& TData, int iter)
        : argsMC(args), TData(TData), currentMotionIter(iter) {}
  };
  void init() override {
    Process::init();
    auto ip = std::dynamic_pointer_cast<InitParameters>(ip_);
    if (!ip) throw std::invalid_argument("GroupwiseRegistration::init: missing InitParameters");
    if (!ip->Dp) throw std::invalid_argument("GroupwiseRegistration::init: null Dp");
    if (ip->lambda.size() != 4) throw std::invalid_argument("GroupwiseRegistration::init: lambda must hold 4 weights");
    auto in = inputAs<XData>("GroupwiseRegistration::init");
    if (in->width() != in->height())
      throw std::invalid_argument("GroupwiseRegistration::init: square frames only (the reference's mask is N x N)");
    prm_.W = ip->W;
    prm_.flagW = ip->flagW ? 1 : 0;
    prm_.radius = int(ip->radius);
    prm_.E = int(ip->E);
    prm_.Dp[0] = ip->Dp[0];
    prm_.Dp[1] = ip->Dp[1];
    prm_.nmax = int(ip->nmax);
    prm_.et = ip->et;
    prm_.eh = ip->eh;
    for (int i = 0; i < 4; ++i) prm_.lambda[i] = ip->lambda[size_t(i)];
    N_ = int(in->width());
    F_ = int(in->getDynDimsTotalSize());
    const int rc = gbn_registration_info_get(N_, F_, &prm_, &info_);
    if (rc == GBN_ERR_INVALID || rc == GBN_ERR_UNSUPPORTED)
      throw std::invalid_argument(std::string("GroupwiseRegistration::init: ") + gbn_last_error_string());
    gbnCheck(rc, "GroupwiseRegistration::init");
    bb_.assign(info_.bound_box, info_.bound_box + 4);
    inited_ = true;
  }
  void launch() override {
    const char* who = "GroupwiseRegistration::launch";
    if (!inited_) throw std::invalid_argument(std::string(who) + ": init() not called");
    auto lp = std::dynamic_pointer_cast<LaunchParameters>(lp_);
    if (!lp || !lp->argsMC) throw std::invalid_argument(std::string(who) + ": missing LaunchParameters or argsMC");
    auto in = inputAs<XData>(who);
    ArgumentsMotionCompensation* a = lp->argsMC;
    const size_t nT = size_t(2) * F_ * info_.cp * info_.cp;
    const float* Tin = nullptr;
    if (lp->TData) {
      if (lp->TData->getBytes() != nT * sizeof(float))
        throw std::invalid_argument(std::string(who) + ": TData must be float [2][F][cp][cp]");
      Tin = static_cast<const float*>(lp->TData->getDevicePtr());
    }
    // fresh outputs: the motion-compensated solve may still hold the previous ones
    auto T = std::make_shared<ArrayData<float>>(app_, nT);
    auto xn = std::make_shared<ArrayData<float>>(app_, size_t(2) * F_ * N_ * N_);
    auto xm = std::make_shared<ArrayData<int>>(app_, size_t(2) * N_ * N_);
    H_.assign(size_t(prm_.nmax) + 1, 0.f);
    gbnCheck(gbn_registration_run(ctx(), static_cast<const float*>(in->getDevicePtr()), N_, F_, &prm_, Tin,
                                  static_cast<float*>(T->getDevicePtr()), static_cast<float*>(xn->getDevicePtr()),
                                  static_cast<int*>(xm->getDevicePtr()), H_.data(), &stats_),
             who);
    H_.resize(size_t(stats_.iterations) + 1);
    a->TData = T;
    a->xnData = xn;
    a->xData = xm;
    a->bound_box = &bb_;
  }
  const gbn_registration_stats& getStats() const { return stats_; }
  /// the metric per iteration (HData of the reference)
  const std::vector<float>& getMetric() const { return H_; }
  int getControlPoints() const { return info_.cp; }

 private:
  gbn_registration_params prm_{};
  gbn_registration_info info_{};
  gbn_registration_stats stats_{};
  std::vector<dimIndexType> bb_;
  std::vector<float> H_;
  int N_ = 0, F_ = 0;
  bool inited_ = false;
};

/// NestaUp (src/processes/nesta/NestaUp.cpp:81-910, NestaUp.hpp:67-83).
class NestaUp : public Process {
 public:
  struct LaunchParameters : Process::LaunchParameters {
    float lambda_i;
    float mu_f;
    float La;
    unsigned int maxIntIter;
    float tolVar;
    int verbose;
    unsigned int maxIter;
    unsigned int stoptest;
    unsigned int miniter;
    ArgumentsMotionCompensation* argsMC;
    bool showProgress;
    LaunchParameters(float lambda_i, float mu_f, float La, unsigned int maxIntIter, float tolVar, int verbose,
                     int maxIter, unsigned int stoptest, unsigned int miniter, ArgumentsMotionCompensation* args,
                     bool sp = false)
        : lambda_i(lambda_i), mu_f(mu_f), La(La), maxIntIter(maxIntIter), tolVar(tolVar), verbose(verbose),
          maxIter(unsigned(maxIter)), stoptest(stoptest), miniter(miniter), argsMC(args), showProgress(sp) {}
  };
  ~NestaUp() override {
    if (prob_) gbn_problem_destroy(prob_);
  }
  void init() override {
    Process::init();
    bind();
  }
  void launch() override {
    auto lp = std::dynamic_pointer_cast<LaunchParameters>(lp_);
    if (!lp) throw std::invalid_argument("NestaUp::launch: missing LaunchParameters");
    bind();
    // with argsMC the sparsity operator is tTV after motion compensation and
    // the solve starts from the output's current image (NestaUp.cpp:201-278, 483-486)
    if (lp->argsMC) {
      auto k = inputAs<KData>("NestaUp");
      const auto m = detail::motion_args(lp->argsMC, k->width(), k->height(), k->getDynDimsTotalSize(),
                                         "NestaUp::launch");
      gbnCheck(gbn_problem_set_motion(prob_, m.xn, m.xmesh, m.bb), "NestaUp::launch");
    } else {
      gbnCheck(gbn_problem_set_motion(prob_, nullptr, nullptr, nullptr), "NestaUp::launch");
    }
    const gbn_nesta_params prm{lp->lambda_i, lp->mu_f, lp->La, lp->maxIntIter, lp->tolVar,
                               lp->verbose, lp->maxIter, lp->stoptest, lp->miniter};
    gbnCheck(gbn_nesta_run(ctx(), prob_, &prm, static_cast<float*>(out_->getDevicePtr()), &stats_), "NestaUp::launch");
    lp->tolVar = stats_.tolVar_final;  // the reference updates LaunchParameters::tolVar in place
  }
  const gbn_nesta_stats& getStats() const { return stats_; }

 private:
  void bind() {
    auto k = inputAs<KData>("NestaUp");
    outputAs<XData>("NestaUp");
    if (!k->getSensitivityMapsData() || !k->getSamplingMasksData())
      throw std::invalid_argument("NestaUp: KData needs sensitivity maps and sampling masks");
    if (prob_ && bound_in_ == in_.get() && bound_k_ == k->getDevicePtr()) return;
    if (prob_) gbn_problem_destroy(prob_);
    prob_ = nullptr;
    gbnCheck(gbn_problem_create(ctx(), int(k->width()), int(k->height()), int(k->getDynDimsTotalSize()),
                                int(k->getNCoils()), static_cast<const float*>(k->getDevicePtr()),
                                static_cast<const float*>(k->getSensitivityMapsData()->getDevicePtr()),
                                static_cast<const uint8_t*>(k->getSamplingMasksData()->getDevicePtr()), &prob_),
             "NestaUp::init");
    bound_in_ = in_.get();
    bound_k_ = k->getDevicePtr();
  }
  gbn_problem* prob_ = nullptr;
  const Data* bound_in_ = nullptr;
  const void* bound_k_ = nullptr;
  gbn_nesta_stats stats_{};
};

}  // namespace OpenCLIPER
