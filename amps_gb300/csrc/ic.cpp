// Host-side initial condition: uniform positions per cell, Maxwellian velocities.
//
// Random numbers come from the reference's multiplicative LCG
// (src/general/rnd.h:56-77: Seed *= 48828125; Seed &= 2^31-1; r = Seed/2^31),
// velocities from the Box-Muller form of test/srcFastWave/main.cpp:282-283,
// v = vth * sqrt(-2 ln(1 - 0.999999999 r1)) * cos(2 pi r2).
//
// The stream is split by block with an exact jump-ahead (Seed_n = Seed_0 * a^n
// mod 2^31), so blocks are generated on several host threads and the result
// does not depend on the thread count.  Draw order inside a block: cells in
// i-fastest order, then the ppc draws of the cell; each draw places one
// particle of every species at the same point (3 position numbers) and then,
// for each axis, the velocity of every species (radius number, angle number).
// Positions and velocities are rounded to FP32 so that FP64 and FP32 consumers
// start from identical particles.
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

#include "../../include/amps_gpu.h"

namespace {

constexpr uint64_t kA = 48828125ULL;
constexpr uint64_t kMask = 2147483647ULL;  // 2^31 - 1

inline uint64_t mulmod31(uint64_t a, uint64_t b) { return (a * b) & kMask; }

uint64_t powmod31(uint64_t a, uint64_t e) {
  uint64_t r = 1, b = a & kMask;
  while (e) {
    if (e & 1) r = mulmod31(r, b);
    b = mulmod31(b, b);
    e >>= 1;
  }
  return r;
}

struct Lcg {
  uint64_t s;
  double next() {
    s = (s * kA) & kMask;
    if (s == 0) s = 1;
    return double(s) / 2147483648.0;
  }
};

float below(float x, float hi) { return x < hi ? x : std::nextafter(hi, 0.0f); }

}  // namespace

extern "C" long long amps_ic_count(int nbx, int nby, int nbz, int ppc, int nspec) {
  if (nbx <= 0 || nby <= 0 || nbz <= 0 || ppc <= 0 || nspec <= 0) return 0;
  return (long long)nbx * nby * nbz * 512LL * ppc * nspec;
}

extern "C" int amps_ic_maxwellian(int nbx, int nby, int nbz, int ppc, int nspec, const double* vth,
                                  unsigned long long seed, int nthreads, float* u, float* v,
                                  uint8_t* spec, int32_t* block) {
  if (nbx <= 0 || nby <= 0 || nbz <= 0 || ppc <= 0 || nspec <= 0 ||
      nspec > AMPS_GPU_MAX_SPECIES || !vth || !u || !v || !spec || !block)
    return AMPS_GPU_INVALID_ARG;
  if ((seed & kMask) == 0) return AMPS_GPU_INVALID_ARG;
  const int nb = nbx * nby * nbz;
  const uint64_t draws_per_block = 512ULL * ppc * (3 + 6ULL * nspec);
  const long long per_block = 512LL * ppc * nspec;
  const uint64_t jump = powmod31(kA, draws_per_block);
  const double two_pi = 6.28318530717958647692528676655900577;

  auto work = [&](int b0, int b1) {
    Lcg g;
    g.s = mulmod31(seed & kMask, powmod31(jump, (uint64_t)b0));
    for (int b = b0; b < b1; b++) {
      long long p = (long long)b * per_block;
      for (int c = 0; c < 512; c++) {
        const int ci = c & 7, cj = (c >> 3) & 7, ck = c >> 6;
        for (int k = 0; k < ppc; k++) {
          float pos[3];
          pos[0] = below((float)((double)ci + g.next()), 8.0f);
          pos[1] = below((float)((double)cj + g.next()), 8.0f);
          pos[2] = below((float)((double)ck + g.next()), 8.0f);
          float vel[AMPS_GPU_MAX_SPECIES][3];
          for (int d = 0; d < 3; d++)
            for (int s = 0; s < nspec; s++) {
              double r1 = g.next();
              double r2 = g.next();
              vel[s][d] = (float)(vth[s] * std::sqrt(-2.0 * std::log(1.0 - .999999999 * r1)) *
                                  std::cos(two_pi * r2));
            }
          for (int s = 0; s < nspec; s++, p++) {
            for (int d = 0; d < 3; d++) {
              u[3 * p + d] = pos[d];
              v[3 * p + d] = vel[s][d];
            }
            spec[p] = (uint8_t)s;
            block[p] = b;
          }
        }
      }
    }
  };

  if (nthreads <= 1 || nb == 1) {
    work(0, nb);
  } else {
    std::vector<std::thread> th;
    int per = (nb + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
      int b0 = t * per, b1 = std::min(nb, b0 + per);
      if (b0 >= b1) break;
      th.emplace_back(work, b0, b1);
    }
    for (auto& t : th) t.join();
  }
  return AMPS_GPU_OK;
}
