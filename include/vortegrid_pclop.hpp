// vortegrid_pclop.hpp -- header-only C++ particle operations over the C ABI
// in vortegrid.h, shaped like the reference's plugin interface so that a
// ParticleGroup can run the GB300 step in place of the CPU one.
//
// Reference interface (mijagourlay/VorteGrid, Samples/MjgIntelFluidDemo_Part20):
//   class IParticleOperation {                       Particles/Operation/particleOperation.h:27-44
//     virtual IParticleOperation* Create() = 0;
//     virtual IParticleOperation* Clone() = 0;
//     virtual void Operate(VECTOR<Particle>& particles, float timeStep, unsigned uFrame) = 0;
//   };
//   class PclOpVortonSim : public IParticleOperation   VortonFluid/pclOpVortonSim.h:46-71
//   { VortonSim mVortonSim; const Vec3* mMinCorner; const Vec3* mMaxCorner; };
//
// This header does not include the reference's headers.  `ParticleVector` is
// any container with data() / size() over records of the reference's Particle
// layout (position at byte 0, velocity at 12, angular velocity at 36, size at
// 52); in the reference, VECTOR<Particle> satisfies it.  `Vec3Like` is any
// type with three contiguous floats (the reference's Vec3).
#ifndef VORTEGRID_PCLOP_HPP
#define VORTEGRID_PCLOP_HPP

#include <stdexcept>
#include <string>

#include "vortegrid.h"

namespace vortegrid {

class Error : public std::runtime_error {
 public:
  Error(vg_status s, const std::string& what) : std::runtime_error(what), status(s) {}
  vg_status status;
};

// Owns one vg_ctx: the GPU counterpart of VortonSim (vortonSim.h:279-455).
class VortonSimGpu {
 public:
  explicit VortonSimGpu(float viscosity = 0.0f, const vg_config* cfg = nullptr) {
    vg_config c;
    if (cfg) {
      c = *cfg;
    } else {
      vg_config_default(&c);
      c.viscosity = viscosity;
    }
    const vg_status s = vg_create(&c, &ctx_);
    if (s != VG_OK) throw Error(s, std::string("vg_create: ") + vg_last_error(nullptr));
  }
  ~VortonSimGpu() { vg_destroy(ctx_); }
  VortonSimGpu(const VortonSimGpu&) = delete;
  VortonSimGpu& operator=(const VortonSimGpu&) = delete;

  vg_ctx* handle() const { return ctx_; }

  // FindBoundingBox + UpdateBoundingBox(extra box, final) + Update(dt, frame).
  template <class ParticleVector, class Vec3Like>
  void Update(ParticleVector& particles, float timeStep, unsigned uFrame, const Vec3Like* minCorner,
              const Vec3Like* maxCorner) {
    check(vg_step(ctx_, particles.data(), particles.size(), sizeof(particles.data()[0]),
                  minCorner ? reinterpret_cast<const float*>(minCorner) : nullptr,
                  maxCorner ? reinterpret_cast<const float*>(maxCorner) : nullptr, timeStep, uFrame),
          "vg_step");
  }

  // Update followed by PclOpEvolve on the same vorton records (vg_step_evolve).
  template <class ParticleVector, class Vec3Like>
  void UpdateAndEvolve(ParticleVector& particles, float timeStep, unsigned uFrame, const Vec3Like* minCorner,
                       const Vec3Like* maxCorner) {
    check(vg_step_evolve(ctx_, particles.data(), particles.size(), sizeof(particles.data()[0]),
                         minCorner ? reinterpret_cast<const float*>(minCorner) : nullptr,
                         maxCorner ? reinterpret_cast<const float*>(maxCorner) : nullptr, timeStep, uFrame),
          "vg_step_evolve");
  }

  // GetVelocityGrid (vortonSim.h:334-335): copies the grid into `xyz`.
  vg_grid_geom GetVelocityGrid(float* xyz, size_t cap_points) {
    vg_grid_geom g;
    check(vg_get_velocity_grid(ctx_, xyz, cap_points, &g), "vg_get_velocity_grid");
    return g;
  }

  // AssignVelocityFromField(gain 1) + Evolve for tracer records.
  template <class ParticleVector>
  void Advect(ParticleVector& tracers, float timeStep) {
    check(vg_advect(ctx_, tracers.data(), tracers.size(), sizeof(tracers.data()[0]), timeStep), "vg_advect");
  }

  vg_step_stats Stats() {
    vg_step_stats s;
    check(vg_get_stats(ctx_, &s), "vg_get_stats");
    return s;
  }

 private:
  void check(vg_status s, const char* what) {
    if (s != VG_OK) throw Error(s, std::string(what) + ": " + vg_last_error(ctx_));
  }
  vg_ctx* ctx_ = nullptr;
};

// Drop-in for PclOpVortonSim.  Base is the caller's IParticleOperation (or any
// class declaring the same virtuals); the template keeps this header free of
// the reference's types.
template <class Base, class ParticleVector, class Vec3Like>
class PclOpVortonSimGpu : public Base {
 public:
  explicit PclOpVortonSimGpu(float viscosity = 0.01f) : mVortonSim(viscosity) {}
  Base* Create() { return new PclOpVortonSimGpu(); }
  Base* Clone() { return new PclOpVortonSimGpu(); }
  // PclOpVortonSim::Operate (pclOpVortonSim.cpp:51-71); with mEvolve, also
  // the PclOpEvolve that follows it on the vorton group, in the same call.
  void Operate(ParticleVector& particles, float timeStep, unsigned uFrame) {
    if (particles.size() == 0) return;  // the reference returns early on no vortons
    if (mEvolve)
      mVortonSim.UpdateAndEvolve(particles, timeStep, uFrame, mMinCorner, mMaxCorner);
    else
      mVortonSim.Update(particles, timeStep, uFrame, mMinCorner, mMaxCorner);
  }
  VortonSimGpu mVortonSim;
  const Vec3Like* mMinCorner = nullptr;
  const Vec3Like* mMaxCorner = nullptr;
  bool mEvolve = false;  // true: drop the vorton group's PclOpEvolve, this op moves the vortons
};

// Drop-in for the tracer group's PclOpAssignVelocityFromField (gain 1) +
// PclOpEvolve pair, reading the velocity grid of a PclOpVortonSimGpu's last
// step (Particles/Operation/pclOpAdvect.cpp:132-152, pclOpEvolve.cpp:36-58).
template <class Base, class ParticleVector>
class PclOpAdvectGpu : public Base {
 public:
  explicit PclOpAdvectGpu(VortonSimGpu* sim = nullptr) : mVortonSim(sim) {}
  Base* Create() { return new PclOpAdvectGpu(); }
  Base* Clone() { return new PclOpAdvectGpu(mVortonSim); }
  void Operate(ParticleVector& particles, float timeStep, unsigned /*uFrame*/) {
    if (mVortonSim && particles.size()) mVortonSim->Advect(particles, timeStep);
  }
  VortonSimGpu* mVortonSim;
};

}  // namespace vortegrid

#endif  // VORTEGRID_PCLOP_HPP
