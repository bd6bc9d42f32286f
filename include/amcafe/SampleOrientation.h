// Drop-in SampleOrientation (reference: src/src-mpi/SampleOrientation.h):
// GenerateSamples (SampleOrientation.C:124-161) draws uniformly distributed
// orientations as (angle, axis) on the host, through the engine's own
// restatement (cafe_generate_samples), which the engine also uses for the
// baseplate and layer grains. See Grid.h.
#ifndef SAMPLEORIENTATION_H
#define SAMPLEORIENTATION_H

#include <vector>

#include "Grid.h"

class SampleOrientation {
 public:
  SampleOrientation() {}
  void GenerateSamples(const int Nsample, unsigned int seedL, std::vector<double> &axisAngle) {
    axisAngle.assign(4 * (size_t)(Nsample > 0 ? Nsample : 0), 0.0);
    amcafe_dropin::check(cafe_generate_samples(Nsample, seedL, axisAngle.data()),
                         "SampleOrientation::GenerateSamples");
  }
};

#endif
