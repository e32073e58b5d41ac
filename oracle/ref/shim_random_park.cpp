/* Oracle shim (test infrastructure only): a drop-in replacement for the
   reference's RandomPark (src/random_park.h:23-36, src/random_park.cpp:35-119).

   While a draw context is open (set by the oracle app and solver subclasses
   in oracle_apps.cpp around one site update or one KMC event), uniform()
   returns the next Philox word of that context as u = (x+1) * 2^-32; in an
   ising sweep both draws come from the site's one word x, the first as
   (2*(x>>31) + 1) / 4 and the second as ((x & 0x7FFFFFFF) + 1) * 2^-31.
   Otherwise it runs the reference's Park-Miller minimal-standard recurrence
   (IA=16807, IM=2^31-1, Schrage factorisation with IQ=127773, IR=2836), so
   that every other consumer (set site range, solver construction) behaves as
   in the unmodified reference.  Only the member layout (public int seed) and
   the method signatures have to match the reference header. */

#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "random_park.h"
#include "shim_ctx.h"

using namespace SPPARKS_NS;

namespace spk_shim {
DrawCtx ctx = {0, {0, 0, 0, 0}, 0, 0, 0, 0};
uint32_t philox_seed = 12345;
uint32_t stream_base = 0;
}  // namespace spk_shim

static const int kIA = 16807;
static const int kIM = 2147483647;
static const double kAM = 1.0 / kIM;
static const int kIQ = 127773;
static const int kIR = 2836;

RandomPark::RandomPark(int iseed) { seed = iseed; }

RandomPark::RandomPark(double rseed) {
  seed = static_cast<int>(rseed * kIM);
  if (seed == 0) seed = 1;
}

void RandomPark::reset(double rseed, int offset, int warmup) {
  seed = static_cast<int>(fmod(rseed * kIM + offset, kIM));
  if (seed < 0) seed = -seed;
  if (seed == 0) seed = 1;
  for (int i = 0; i < warmup; i++) uniform();
}

void RandomPark::tagreset(double rseed, tagint offset, int warmup) {
  seed = static_cast<int>(fmod(rseed * kIM + offset, kIM));
  if (seed < 0) seed = -seed;
  if (seed == 0) seed = 1;
  for (int i = 0; i < warmup; i++) uniform();
}

double RandomPark::uniform() {
  spk_shim::DrawCtx &c = spk_shim::ctx;
  if (c.active) {
    if (c.next >= c.limit) {
      fprintf(stderr, "oracle shim: draw %d requested, context allows %d\n", c.next, c.limit);
      exit(3);
    }
    if (c.ising) {
      uint32_t x = c.w[c.base];
      return c.next++ == 0 ? (2.0 * (double)(x >> 31) + 1.0) * 0.25
                           : ((double)(x & 0x7FFFFFFFu) + 1.0) * (1.0 / 2147483648.0);
    }
    uint32_t x = c.w[c.base + c.next];
    c.next++;
    return ((double)x + 1.0) * (1.0 / 4294967296.0);
  }
  int k = seed / kIQ;
  seed = kIA * (seed - k * kIQ) - kIR * k;
  if (seed < 0) seed += kIM;
  return kAM * seed;
}

int RandomPark::irandom(int n) {
  int i = (int)(uniform() * n) + 1;
  if (i > n) i = n;
  return i;
}

tagint RandomPark::tagrandom(tagint n) {
  tagint i = (tagint)(uniform() * n) + 1;
  if (i > n) i = n;
  return i;
}

bigint RandomPark::bigrandom(bigint n) {
  bigint i = (bigint)(uniform() * n) + 1;
  if (i > n) i = n;
  return i;
}
