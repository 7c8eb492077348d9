// Host stand-in for the reference's OpenCLIPER/kernels/hostKernelFunctions.h
// -- TEST INFRASTRUCTURE (oracle).  It lets the reference's own .cl kernels and
// dims/strides accessors (src/kernels/hostKernelFunctions.cl) compile as C++
// on the host: OpenCL C address-space keywords and built-ins are mapped to
// plain C++, and the accessor interface is restated (same struct layout and
// enum values as include/OpenCLIPER/kernels/hostKernelFunctions.h and
// include/OpenCLIPER/kernels/defs.h).
#ifndef GBN_REF_HOSTKERNELFUNCTIONS_H
#define GBN_REF_HOSTKERNELFUNCTIONS_H

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

typedef uint32_t cl_uint;
typedef unsigned char uchar;
typedef float realType;

#define global
#define __global
#define kernel
#define __kernel
#define __const const
#define dimIndexType cl_uint
#define PRINTF(x) do {} while (0)

// OpenCL C vector types used by the kernels
struct float2 {
  float x, y;
  float2() : x(0.f), y(0.f) {}
  float2(float a, float b) : x(a), y(b) {}
  float2(int s) : x(float(s)), y(float(s)) {}  // scalar broadcast, e.g. `acum = 0`
  float2& operator+=(const float2& o) { x += o.x; y += o.y; return *this; }
};
inline float2 operator+(float2 a, float2 b) { return float2(a.x + b.x, a.y + b.y); }
inline float2 operator-(float2 a, float2 b) { return float2(a.x - b.x, a.y - b.y); }
inline float2 operator/(float2 a, float s) { return float2(a.x / s, a.y / s); }
inline float2 operator*(float2 a, float s) { return float2(a.x * s, a.y * s); }
inline float2 operator*(float s, float2 a) { return float2(s * a.x, s * a.y); }
struct uint2 {
  cl_uint x, y;
};
typedef float2 complexType;

// work-item id and global sizes of the NDRange being executed by the host harness
extern thread_local size_t gbnref_gid[3];
extern thread_local size_t gbnref_gsz[3];
inline size_t get_global_id(int d) { return gbnref_gid[d]; }
inline size_t get_global_size(int d) { return gbnref_gsz[d]; }
// the harness runs work-items one after another, so compare-and-swap is plain
inline cl_uint atomic_cmpxchg(volatile cl_uint* p, cl_uint cmp, cl_uint val) {
  const cl_uint old = *p;
  if (old == cmp) *p = val;
  return old;
}
inline float length(float2 v) { return std::sqrt(v.x * v.x + v.y * v.y); }
inline float as_float(cl_uint u) { float f; std::memcpy(&f, &u, 4); return f; }
inline cl_uint as_uint(float f) { cl_uint u; std::memcpy(&u, &f, 4); return u; }

enum DimsPos { WIDTHPOS = 0, HEIGHTPOS = 1, DEPTHPOS = 2 };
#define NUMINITIALPOSITIONSDIMSINFO 4
enum knownDimPos { NumSpatialDimsPos = 0, AllSizesEqualPos = 1, NumCoilsPos = 2, NumTemporalDimsPos = 3, FirstTemporalDimPos = 4 };
enum knownStridePos { ElementStridePos = 0, FirstSpatialStridePos = 0 };
enum knownSpatialDimPos { COLUMNS = WIDTHPOS, ROWS = HEIGHTPOS, SLICES = DEPTHPOS };

struct __attribute__((packed)) dimsAndStridesKnownFields {
  cl_uint numSpatialDims;
  cl_uint allSizesEqual;
  cl_uint numCoils;
  cl_uint numTemporalDims;
  cl_uint firstTemporalDimSize;
};

extern "C" {
cl_uint roundUp(cl_uint numToRound, cl_uint baseNumber);
cl_uint getDimsAndStridesArrayOffsetInBytes(const void* buffer);
const cl_uint* getDimsAndStridesArrayInBuffer(const void* buffer);
const struct dimsAndStridesKnownFields* getDimsAndStridesStruct(const void* buffer);
const cl_uint* getStridesArray(const void* buffer);
cl_uint getNumSpatialDims(const void* buffer);
cl_uint getNumNDArrays(const void* buffer);
cl_uint getNDArray1DIndex(const void* buffer, cl_uint coilIndex, cl_uint temporalDimIndexes[]);
cl_uint getNDArrayTotalSize(const void* buffer, cl_uint NDArray1DIndex);
cl_uint getNDArrayStride(const void* buffer);
cl_uint getSpatialDimStride(const void* buffer, cl_uint spatialDimIndex, cl_uint NDArray1DIndex);
cl_uint getSpatialDimSize(const void* buffer, cl_uint spatialDimIndex, cl_uint NDArray1DIndex);
cl_uint getNumCoils(const void* buffer);
cl_uint getCoilDim(const void* buffer);
cl_uint getCoilStride(const void* buffer, cl_uint NDArray1DIndex);
cl_uint getNumTemporalDims(const void* buffer);
cl_uint getTemporalDim(const void* buffer, cl_uint tempDim);
cl_uint getTemporalDimStride(const void* buffer, cl_uint temporalDimIndex, cl_uint NDArray1DIndex);
cl_uint getTemporalDimSize(const void* buffer, cl_uint temporalDimIndex);
cl_uint getDimSize(const void* buffer, cl_uint dimIndex, cl_uint NDArray1DIndex);
cl_uint getElementStride(const void* buffer, cl_uint NDArray1DIndex);
cl_uint getDimStride(const void* buffer, cl_uint dimIndex, cl_uint NDArray1DIndex);
const void* getNextElement(const void* buffer, cl_uint dimIndex, cl_uint curNDArray, cl_uint curOffset);
}

#endif
