// Single-particle wakes of the reference (Wake::singleWakeResistive, singleWakeGeometric,
// singleWakeRoughness, src/Main/Wake.cpp:140-434) called directly, for known-answer
// vectors. Those members are private and need the &wake namelist, Time, Setup and
// Profile objects to reach through Wake::init; this translation unit of the checker
// opens the class instead, so that only the three computations run.
// Wake.h's own includes first, so that only the Wake class is opened
#include <complex>
#include <iostream>
#include <string>
#include <vector>

#include "GenProfile.h"
#include "GenTime.h"
#include "Particle.h"
#include "Setup.h"
#include "StringProcessing.h"
#define private public
#include "Wake.h"
#undef private

extern "C" void g4ref_single_wakes(int ns, double ds, double radius, double conductivity, double relaxation,
                                   int roundpipe, double gap, double lgap, double hrough, double lrough,
                                   double *res, double *geo, double *rou) {
  Wake w;
  w.ns = static_cast<unsigned>(ns);
  w.ds = ds;
  w.radius = radius;
  w.conductivity = conductivity;
  w.relaxation = relaxation;
  w.roundpipe = roundpipe != 0;
  w.gap = gap;
  w.lgap = lgap;
  w.hrough = hrough;
  w.lrough = lrough;
  w.wakeres = res;
  w.wakegeo = geo;
  w.wakerou = rou;
  // rank 1: the reference prints its progress on rank 0 only
  w.singleWakeResistive(1);
  w.singleWakeGeometric(1);
  w.singleWakeRoughness(1);
  w.wakeres = w.wakegeo = w.wakerou = nullptr;
}
