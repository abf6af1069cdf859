// Stand-in for exaDEM's contact_parameters.hpp, which needs yaml-cpp: only the
// plain parameter record the contact law reads, with the field names of
// src/forcefield/include/exaDEM/forcefield/contact_parameters.hpp:32-41.
#pragma once
#include <onika/log.h>
namespace exaDEM {
struct ContactParams {
  double kn_ = 0;
  double kt_ = 0;
  double kr_ = 0;
  double mu_ = 0;
  double damp_rate_ = 0;
  double fc_ = 0;
  double dncut_ = 0;
  double gamma_ = 0;
};
}  // namespace exaDEM
