// Host helpers shared by the mesh generator and the device mesh context.
#include "common.hh"

namespace mpaso {

static thread_local std::string g_last_error;

void set_last_error(const std::string &msg) { g_last_error = msg; }

uint64_t hilbert_key(const uint32_t *coords, int dims, int bits) {
  uint32_t x[3] = {0, 0, 0};
  for (int i = 0; i < dims; ++i) x[i] = coords[i];
  const uint32_t top = 1u << (bits - 1);
  // Undo excess work: for each bit plane from the top, either invert the low
  // bits of x[0] or exchange them with x[i] (Skilling 2004, AxestoTranspose).
  for (uint32_t q = top; q > 1; q >>= 1) {
    const uint32_t p = q - 1;
    for (int i = 0; i < dims; ++i) {
      if (x[i] & q) {
        x[0] ^= p;
      } else {
        const uint32_t t = (x[0] ^ x[i]) & p;
        x[0] ^= t;
        x[i] ^= t;
      }
    }
  }
  // Gray encode.
  for (int i = 1; i < dims; ++i) x[i] ^= x[i - 1];
  uint32_t t = 0;
  for (uint32_t q = top; q > 1; q >>= 1)
    if (x[dims - 1] & q) t ^= q - 1;
  for (int i = 0; i < dims; ++i) x[i] ^= t;
  // Interleave the transposed bits, most significant plane first.
  uint64_t key = 0;
  for (int b = bits - 1; b >= 0; --b)
    for (int i = 0; i < dims; ++i) key = (key << 1) | ((x[i] >> b) & 1u);
  return key;
}

uint64_t morton_key(const uint32_t *coords, int dims, int bits) {
  uint64_t key = 0;
  for (int b = bits - 1; b >= 0; --b)
    for (int i = 0; i < dims; ++i) key = (key << 1) | ((coords[i] >> b) & 1u);
  return key;
}

}  // namespace mpaso

extern "C" const char *mpaso_last_error(void) { return mpaso::g_last_error.c_str(); }
