// Project-written stand-in for MCBooster's PhaseSpace generator.  It does not generate: Generate() takes the
// events a caller handed to SetGeneratedEvents (n events of k daughters, (E, px, py, pz) each), all accepted
// with unit weight, so that the reference's amplitude PDFs see exactly the phase-space events the engine and
// the FP64 restatement are given.  Without supplied events Generate() throws.
#pragma once
#include <mcbooster/GContainers.h>
#include <stdexcept>
#include <vector>

namespace mcbooster {
void SetGeneratedEvents(const GReal_t *p4, GLong_t n, GInt_t ndaughters);

class PhaseSpace {
  public:
    PhaseSpace(GReal_t motherMass, std::vector<GReal_t> masses, GLong_t n, GLong_t offset = 0)
        : nreq_(n), masses_(masses) {
        (void)motherMass;
        (void)offset;
    }
    void Generate(const Vector4R &mother);
    void Unweight() {}
    GLong_t GetNAccepted() const { return (GLong_t)(daughters_.empty() ? 0 : daughters_[0].size()); }
    BoolVector_d GetAccRejFlags() const { return BoolVector_d(GetNAccepted(), true); }
    RealVector_d GetWeights() const { return RealVector_d(GetNAccepted(), 1.0); }
    Particles_d &GetDaughters(int i) { return daughters_.at(i); }
    void SetSeed(GInt_t s) { seed_ = s; }
    GInt_t GetSeed() const { return seed_; }
    void FreeResources() { daughters_.clear(); }

  private:
    GLong_t nreq_;
    std::vector<GReal_t> masses_;
    std::vector<Particles_d> daughters_;
    GInt_t seed_ = 0;
};
} // namespace mcbooster
