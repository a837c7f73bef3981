// Test infrastructure only: correctly rounded f32 sin, cos, asin and atan2
// for the CPU oracle.  Only tests/, __graft_entry__.smoke() and the bench's
// CPU-baseline leg may load anything built from oracle/.
//
// The reference calls the platform's f32 libm through Rust std (f32::sin_cos,
// asin, atan2: crates/physics/src/avbd/rows.rs:115, :145,
// crates/physics/src/sequential_impulse/joints.rs:46).  A correctly rounded
// result is the one float nearest the exact value, so it does not depend on
// the library that computes it.  The oracle takes it from the host build of
// the device's implementation (ornis_gb300/csrc/avbd_crmath.cuh: a float
// stage, a double stage and a double-double stage, each with Ziv's rounding
// test), which runs at libm speed on the host, so the timed CPU baseline is
// not slowed by it.  Its correctness is checked independently: the host
// build against the long-double functions rounded once to float over argument
// sweeps of about 40 M arguments (tests/test_crmath_cpu.py), in builds that
// force each stage.  f64 worlds keep std's double functions.
#pragma once
#include <cmath>

#include "../ornis_gb300/csrc/avbd_crmath.cuh"

namespace orc {

inline float osin(float x) { return avbd::crm::sinf(x); }
inline float ocos(float x) { return avbd::crm::cosf(x); }
inline float oasin(float x) { return avbd::crm::asinf(x); }
inline float oatan2(float y, float x) { return avbd::crm::atan2f(y, x); }
inline double osin(double x) { return std::sin(x); }
inline double ocos(double x) { return std::cos(x); }
inline double oasin(double x) { return std::asin(x); }
inline double oatan2(double y, double x) { return std::atan2(y, x); }

}  // namespace orc
