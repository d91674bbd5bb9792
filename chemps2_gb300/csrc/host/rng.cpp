#include "rng.hpp"

#include <cstdlib>

namespace c2g {

HostRand::HostRand(unsigned seed) : own_(true) {
  int32_t r[34];
  r[0] = static_cast<int32_t>(seed == 0 ? 1u : seed);
  for (int i = 1; i < 31; i++) {
    // 16807 * r mod (2^31 - 1) without overflow (Schrage: 2^31 - 1 = 16807 * 127773 + 2836)
    const int32_t hi = r[i - 1] / 127773, lo = r[i - 1] % 127773;
    int32_t w = 16807 * lo - 2836 * hi;
    if (w < 0) w += 2147483647;
    r[i] = w;
  }
  for (int i = 0; i < 31; i++) ring_[i] = static_cast<uint32_t>(r[i]);
  // r[31..33] repeat r[0..2]; the ring then holds r[i-31 .. i-1] at i = 34
  pos_ = 0;
  uint32_t tail[3] = {ring_[0], ring_[1], ring_[2]};
  for (int i = 0; i < 28; i++) ring_[i] = ring_[i + 3];
  ring_[28] = tail[0];
  ring_[29] = tail[1];
  ring_[30] = tail[2];
  for (int i = 0; i < 310; i++) next();
}

int HostRand::next() {
  if (!own_) return std::rand();
  // ring_[pos_] is r[i-31]; r[i-3] sits 28 places further on
  const uint32_t v = ring_[pos_] + ring_[(pos_ + 28) % 31];
  ring_[pos_] = v;
  pos_ = (pos_ + 1) % 31;
  return static_cast<int>(v >> 1);
}

double HostRand::unit() { return static_cast<double>(next()) / RAND_MAX; }

}  // namespace c2g
