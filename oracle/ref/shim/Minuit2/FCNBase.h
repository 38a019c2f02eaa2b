// Project-written stand-ins for the Minuit2 types that the reference's fit headers name
// (include/goofit/fitting/{FCN,Params,FitManagerMinuit2}.h).  Minuit2 is an empty submodule of the
// reference; nothing built here minimises, so these carry no algorithm.
#pragma once
#include <string>
#include <vector>

namespace ROOT {
namespace Minuit2 {
class FCNBase {
  public:
    virtual ~FCNBase() = default;
    virtual double operator()(const std::vector<double> &) const = 0;
    virtual double Up() const = 0;
    virtual double ErrorDef() const { return Up(); }
};
class MnUserParameters {
  public:
    MnUserParameters() = default;
    bool Add(const std::string &, double, double) { return true; }
    bool Add(const std::string &, double, double, double, double) { return true; }
    bool Add(const std::string &, double) { return true; }
};
class MnUserParameterState {
  public:
    MnUserParameterState() = default;
    double Value(unsigned int) const { return 0; }
    double Error(unsigned int) const { return 0; }
};
class FunctionMinimum {
  public:
    bool IsValid() const { return false; }
};
class MnScan {};
} // namespace Minuit2
} // namespace ROOT
