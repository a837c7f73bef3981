// Test infrastructure only: correctly rounded f32 sin, cos, asin and atan2
// for the CPU oracle.  Only tests/, __graft_entry__.smoke() and the bench's
// CPU-baseline leg may load anything built from oracle/.
//
// The reference calls the platform's f32 libm through Rust std (f32::sin_cos,
// asin, atan2: crates/physics/src/avbd/rows.rs:115, :145,
// crates/physics/src/sequential_impulse/joints.rs:46).  A correctly rounded
// result is the one float nearest the exact value, so it does not depend on
// the library that computes it; the oracle computes it as the long-double
// function (x86: 64-bit significand, about 2^-63 relative error; aarch64:
// IEEE quad) rounded once to float, which for float arguments is the
// correctly rounded float except for arguments whose value lies within about
// 2^-60 of a midpoint between two floats (none is known for these functions;
// the device's double / double-double implementation is checked against
// this one over argument sweeps).  f64 worlds keep std's double functions.
#pragma once
#include <cmath>

namespace orc {

inline float osin(float x) { return (float)sinl((long double)x); }
inline float ocos(float x) { return (float)cosl((long double)x); }
inline float oasin(float x) { return (float)asinl((long double)x); }
inline float oatan2(float y, float x) { return (float)atan2l((long double)y, (long double)x); }
inline double osin(double x) { return std::sin(x); }
inline double ocos(double x) { return std::cos(x); }
inline double oasin(double x) { return std::asin(x); }
inline double oatan2(double y, double x) { return std::atan2(y, x); }

}  // namespace orc
