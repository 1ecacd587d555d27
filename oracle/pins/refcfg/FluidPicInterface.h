// Hand-written stand-ins for the SWMF coupler types the reference headers
// name (absent from the reference tree); none of them is called by the pinned
// functions.
#pragma once
#include "pin_config.h"
#include <string>
#include <vector>
#include <array>
class FluidPicInterface {
 public:
  template <class... A> double getPICP(A...) { return 0; }
  template <class... A> double getPICPpar(A...) { return 0; }
  template <class... A> double getPICUth(A...) { return 0; }
  template <class... A> double getPICUx(A...) { return 0; }
  template <class... A> double getPICUy(A...) { return 0; }
  template <class... A> double getPICUz(A...) { return 0; }
  template <class... A> double getBx(A...) { return 0; }
  template <class... A> double getBy(A...) { return 0; }
  template <class... A> double getBz(A...) { return 0; }
};
class Writer {};
class VectorPointList {};
template <class T> class MDArray {};
struct cStubNorm { double norm[3]; };
class cInternalSphericalData_UserDefined {
 public:
  double* SamplingBuffer = nullptr;
  double** SurfaceElementPopulation = nullptr;
  cStubNorm* SurfaceElementExternalNormal = nullptr;
  double* SurfaceElementArea = nullptr;
  double* SolarWindSurfaceFlux = nullptr;
  template <class... A> int ParticleSphereInteraction(A...) { return 0; }
};
class cInternalRotationBodyData_UserDefined {};
class cInternalNastranSurfaceData_UserDefined {};
