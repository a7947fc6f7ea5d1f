// Drives PclOpVortonSimGpu exactly as the reference's ParticleGroup drives its
// operations (Particles/particleGroup.cpp:71-83): a vorton group with the GPU
// VortonSim operation, then a tracer group advected through its velocity grid.
// Reads a binary file of Particle records (argv[1]), runs one step, writes
// the updated records to argv[2].  Used by tests/test_gpu_cpp.py.
#include <cstdio>
#include <cstring>
#include <vector>

#include "vortegrid_pclop.hpp"

struct Vec3 { float x, y, z; };
struct Particle {  // the reference's Particle record on LP64 (Particles/particle.h:425-482)
  Vec3 mPosition, mVelocity, mOrientation, mAngularVelocity;
  float mDensity, mSize;
  int mBirthTime;
  float mFuelFraction, mFlameFraction, mSmokeFraction;
  float mSiblingFields[6];
};
static_assert(sizeof(Particle) == 96, "Particle record must be 96 bytes");

class IParticleOperation {  // Particles/Operation/particleOperation.h:27-44
 public:
  virtual ~IParticleOperation() {}
  virtual IParticleOperation* Create() = 0;
  virtual IParticleOperation* Clone() = 0;
  virtual void Operate(std::vector<Particle>& particles, float timeStep, unsigned uFrame) = 0;
};

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 3;
  std::vector<Particle> vortons;
  Particle p;
  while (fread(&p, sizeof(p), 1, f) == 1) vortons.push_back(p);
  fclose(f);
  typedef vortegrid::PclOpVortonSimGpu<IParticleOperation, std::vector<Particle>, Vec3> Op;
  Op* op = new Op(0.01f);
  Vec3 lo = {-1.5f, -1.5f, -1.0f}, hi = {1.5f, 1.5f, 1.0f};
  op->mMinCorner = &lo;
  op->mMaxCorner = &hi;
  std::vector<IParticleOperation*> ops(1, op);
  try {
    for (IParticleOperation* o : ops) o->Operate(vortons, 1.0f / 30.0f, 0);
    std::vector<Particle> tracers(1000);
    for (size_t i = 0; i < tracers.size(); ++i) {
      std::memset(&tracers[i], 0, sizeof(Particle));
      tracers[i].mPosition = {-1.0f + 2.0f * (i % 10) / 10.0f, -1.0f + 2.0f * ((i / 10) % 10) / 10.0f,
                              -0.5f + 1.0f * (i / 100) / 10.0f};
    }
    vortegrid::PclOpAdvectGpu<IParticleOperation, std::vector<Particle> > adv(&op->mVortonSim);
    adv.Operate(tracers, 1.0f / 30.0f, 0);
    vg_step_stats st = op->mVortonSim.Stats();
    printf("grid %u %u %u cycles %d relres %.3e\n", st.grid.num_points[0], st.grid.num_points[1],
           st.grid.num_points[2], st.poisson_cycles, st.poisson_relres);
  } catch (const vortegrid::Error& e) {
    fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  f = fopen(argv[2], "wb");
  fwrite(vortons.data(), sizeof(Particle), vortons.size(), f);
  fclose(f);
  delete op;
  return 0;
}
