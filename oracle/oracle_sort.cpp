// ORACLE — test infrastructure only (see oracle_math.h).  CPU restatement of
// the reference's photon-beam ordering:
//   split_pass : one stable 1-bit split by a Blelloch scan of the "false"
//                flags, as tests::radixSort does it (Tests.cpp:133-223, 256
//                "threads" x 4 elements, n padded to a power of two) and as
//                calculateScatterOffsets does on the GPU
//                (PPB_RadixSort_LocalSort.comp:70-149)
//   local_sort : one work group's 4-bit sort = four 1-bit splits
//                (PPB_RadixSort_LocalSort.comp:154-220)
//   lsd_sort   : the pipeline the reference intended per 4-bit digit —
//                LocalSort per 1024-key block, 16-bin block histograms laid
//                out digit-major (histogram[digit * #WG + wg]; the shader
//                omits "+ wg", LocalSort.comp:250), an exclusive scan
//                (PrefixSum.comp, serial and wrong as shipped), and the
//                global scatter (GlobalSort.comp, bounds wrong as shipped).
//   morton     : expandBits / getMortonCode (PPB_PT.comp:317-333), 24-bit,
//                and the 30-bit variant over the cloud box.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

namespace oracle {

// tests::radixSort restated: stable split of keys[0..n) on bit `shift`
// (n <= 1024).  Returns the scatter offsets too.
static void split_pass(std::vector<uint32_t>& keys, std::vector<uint32_t>& vals, uint32_t shift) {
  const size_t n = keys.size();
  if (n <= 1) return;
  size_t count = 1;
  while (count < n) count <<= 1;  // pow(2, ceil(log2(n)))
  std::vector<uint32_t> falses(count, 0u), scatter(n);
  for (size_t i = 0; i < n; ++i) {
    falses[i] = ((keys[i] >> shift) & 1u) ^ 1u;
    scatter[i] = falses[i];
  }
  // up-sweep: falses[offset(2i+2)-1] += falses[offset(2i+1)-1] for i < d
  size_t offset = 1;
  for (size_t d = count >> 1; d > 0; d >>= 1) {
    for (size_t i = 0; i < d; ++i) {
      size_t ai = offset * (2 * i + 1) - 1, bi = offset * (2 * i + 2) - 1;
      falses[bi] += falses[ai];
    }
    offset *= 2;
  }
  uint32_t total = falses[count - 1];
  falses[count - 1] = 0;
  // down-sweep
  for (size_t d = 1; d < count; d *= 2) {
    offset >>= 1;
    for (size_t i = 0; i < d; ++i) {
      size_t ai = offset * (2 * i + 1) - 1, bi = offset * (2 * i + 2) - 1;
      uint32_t t = falses[ai];
      falses[ai] = falses[bi];
      falses[bi] += t;
    }
  }
  std::vector<uint32_t> k2(n), v2(n);
  for (size_t i = 0; i < n; ++i) {
    uint32_t pos = scatter[i] == 0u ? (uint32_t)(i - falses[i] + total) : falses[i];
    k2[pos] = keys[i];
    v2[pos] = vals[i];
  }
  keys.swap(k2);
  vals.swap(v2);
}

// A digit of `width` (<= 4) bits from base_shift up: one 1-bit split pass
// per bit (LocalSort.comp:154-252 runs four); a last digit narrower than 4
// bits keeps bits at or above the sort's end out of the order.
static void local_sort(std::vector<uint32_t>& keys, std::vector<uint32_t>& vals, uint32_t base_shift,
                       uint32_t width) {
  for (uint32_t b = 0; b < width; ++b) split_pass(keys, vals, base_shift + b);
}

}  // namespace oracle

using namespace oracle;

extern "C" {

// The Tests.cpp:113-131 fixture: 176 keys from std::mt19937(1) through
// std::uniform_int_distribution(0, 255) (this build's standard library;
// the reference was built with MSVC's, whose distribution may differ).
void oracle_sort_fixture_keys(uint32_t* out) {
  std::mt19937 gen(1);
  std::uniform_int_distribution<int> dist(0, 255);
  for (int i = 0; i < 176; ++i) out[i] = (uint32_t)dist(gen);
}

// tests::localSort: eight 1-bit split passes over the fixture (bit 0..7).
void oracle_split_sort(uint32_t* keys, uint32_t n, uint32_t first_bit, uint32_t nbits) {
  std::vector<uint32_t> k(keys, keys + n), v(n);
  for (uint32_t i = 0; i < n; ++i) v[i] = i;
  for (uint32_t b = 0; b < nbits; ++b) split_pass(k, v, first_bit + b);
  std::copy(k.begin(), k.end(), keys);
}

// The intended reference pipeline for bits [begin, end), 4 bits per pass.
void oracle_lsd_sort_pairs(const uint32_t* kin, const uint32_t* vin, uint32_t n, uint32_t begin, uint32_t end,
                           uint32_t* kout, uint32_t* vout) {
  const uint32_t wg = 1024;  // ELEMENTS_PER_WORK_GROUP (LocalSort.comp:50-51)
  std::vector<uint32_t> k(kin, kin + n), v(n);
  for (uint32_t i = 0; i < n; ++i) v[i] = vin ? vin[i] : i;
  for (uint32_t shift = begin; shift < end; shift += 4) {
    const uint32_t width = std::min(4u, end - shift);
    const uint32_t dmask = (1u << width) - 1u;
    uint32_t groups = (n + wg - 1) / wg;
    std::vector<uint32_t> hist((size_t)16 * groups, 0u);
    std::vector<uint32_t> lk(n), lv(n);
    for (uint32_t g = 0; g < groups; ++g) {
      uint32_t a = g * wg, b = std::min(n, a + wg);
      std::vector<uint32_t> bk(k.begin() + a, k.begin() + b), bv(v.begin() + a, v.begin() + b);
      local_sort(bk, bv, shift, width);
      for (uint32_t i = 0; i < b - a; ++i) {
        lk[a + i] = bk[i];
        lv[a + i] = bv[i];
        hist[(size_t)((bk[i] >> shift) & dmask) * groups + g] += 1;  // digit-major
      }
    }
    // exclusive scan of the digit-major histogram
    std::vector<uint32_t> scan(hist.size());
    uint32_t run = 0;
    for (size_t i = 0; i < hist.size(); ++i) {
      scan[i] = run;
      run += hist[i];
    }
    // global scatter: offset(digit, group) + rank inside the group's run
    for (uint32_t g = 0; g < groups; ++g) {
      uint32_t a = g * wg, b = std::min(n, a + wg);
      uint32_t seen[16] = {0};
      for (uint32_t i = a; i < b; ++i) {
        uint32_t d = (lk[i] >> shift) & dmask;
        uint32_t o = scan[(size_t)d * groups + g] + seen[d]++;
        k[o] = lk[i];
        v[o] = lv[i];
      }
    }
    (void)lk;
  }
  std::copy(k.begin(), k.end(), kout);
  std::copy(v.begin(), v.end(), vout);
}

static uint32_t expand_bits(uint32_t v) {  // PPB_PT.comp:319-325 (+ the 10-bit first step)
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

void oracle_morton(const float* pts, uint32_t n, const float* b0, const float* b1, uint32_t bits, uint32_t* out) {
  for (uint32_t i = 0; i < n; ++i) {
    float p[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    uint32_t q[3];
    for (int a = 0; a < 3; ++a) {
      if (bits == 24) {
        float r = p[a] - b0[a];
        q[a] = (uint32_t)std::fmin(std::fmax(r / 256.0f, 0.0f), 255.0f);
      } else {
        float x = ((p[a] - b0[a]) / (b1[a] - b0[a])) * 1024.0f;
        x = std::fmin(std::fmax(x, 0.0f), 1023.0f);
        q[a] = (uint32_t)x;
      }
    }
    out[i] = (expand_bits(q[0]) << 2) + (expand_bits(q[1]) << 1) + expand_bits(q[2]);
  }
}

}  // extern "C"
