// Host-side check of the line kernel's shared-memory plan and of the bulk
// neighbour-copy windows (no kernel runs): for every dimension, points per
// line, stage-input type and cells per block, the neighbour area is 16-byte
// aligned and large enough for both the per-thread line slots and the bulk
// slots, and every window of a neighbour's field array is 16-byte aligned,
// a multiple of 16 bytes, contains the array and fits its slot.
#include <cstdio>

#include "../../exwave_gb300/csrc/ew_cart.cuh"

using namespace ew;

static int failures = 0;

template <int DIM, int NP, typename Real, typename InT>
void check() {
  constexpr int N = ipow_c(NP, DIM);
  constexpr int F = DIM + 1;
  constexpr int NL = ipow_c(NP, DIM - 1);
  constexpr int SLOT = CartSmem<DIM, NP, Real, InT>::NB_SLOT;
  const size_t fbytes = (size_t)N * sizeof(InT);
  for (int cb = 1; cb * DIM * NL <= 1024; ++cb)
    for (int sx = 0; sx < 2; ++sx)
      for (int sa = 0; sa < 2; ++sa) {
        const CartSmem<DIM, NP, Real, InT> lay(cb, sx != 0, sa != 0);
        const size_t lines = (size_t)cb * DIM * NL * 4 * NP * sizeof(InT);
        const size_t slots = (size_t)cb * 2 * DIM * 2 * SLOT;
        bool ok = lay.nb % 16 == 0 && lay.end >= lay.nb + lines;
        if (cart_nb_bulk<DIM, NP, InT>()) ok = ok && SLOT % 16 == 0 && lay.end >= lay.nb + slots;
        if (!ok) {
          std::printf("FAIL layout dim %d np %d in %zu cb %d\n", DIM, NP, sizeof(InT), cb);
          ++failures;
        }
      }
  if (!cart_nb_bulk<DIM, NP, InT>()) return;
  // windows, for arrays whose cell stride is a multiple of 16 bytes (the
  // condition under which the host enables bulk copies)
  if ((size_t)F * fbytes % 16 != 0) return;
  for (long nb = 0; nb < 4096; ++nb)
    for (int f = 0; f < F; ++f) {
      const size_t s0 = ((size_t)nb * F + f) * fbytes;
      const size_t w0 = s0 & ~(size_t)15;
      const size_t len = ((s0 + fbytes + 15) & ~(size_t)15) - w0;
      const size_t rem = s0 & 15;
      const size_t end_of_array = (size_t)(nb + 1) * F * fbytes;
      if (w0 % 16 || len % 16 || rem + fbytes > len || len > (size_t)SLOT || w0 + len > end_of_array ||
          rem % sizeof(InT)) {
        std::printf("FAIL window dim %d np %d in %zu nb %ld f %d\n", DIM, NP, sizeof(InT), nb, f);
        ++failures;
        return;
      }
    }
}

template <int DIM, int NP>
void check_np() {
  check<DIM, NP, float, float>();
  check<DIM, NP, float, double>();
  check<DIM, NP, double, double>();
  check<DIM, NP, FF, FF>();
  check<DIM, NP, FF, double>();
}

int main() {
  check_np<2, 2>(); check_np<2, 3>(); check_np<2, 4>(); check_np<2, 5>();
  check_np<2, 6>(); check_np<2, 7>(); check_np<2, 8>(); check_np<2, 9>(); check_np<2, 10>();
  check_np<2, 11>(); check_np<2, 12>(); check_np<2, 13>();
  check_np<3, 2>(); check_np<3, 3>(); check_np<3, 4>(); check_np<3, 5>();
  check_np<3, 6>(); check_np<3, 7>(); check_np<3, 8>();
  if (failures) return 1;
  std::printf("OK\n");
  return 0;
}
