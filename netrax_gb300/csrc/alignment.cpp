// Alignment front end: character -> state-mask encoding and pattern
// compression, the two steps between an alignment file and netlk_create
// (raxml-ng performs them through libpll before NetRAX builds its
// partitions: opts.use_pattern_compression, src/RaxmlWrapper.cpp:329-330).
#include <cstdint>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/netlk.h"

namespace netlk {
void set_global_error(const std::string &msg);
}

namespace {

// DNA, bit i = state i in the order A C G T; IUPAC ambiguity codes are the
// unions of their bases; N ? - . O X are every state.
uint32_t dna_mask(char ch) {
  switch (ch >= 'a' && ch <= 'z' ? (char)(ch - 32) : ch) {
    case 'A': return 1u;
    case 'C': return 2u;
    case 'G': return 4u;
    case 'T': case 'U': return 8u;
    case 'R': return 1u | 4u;
    case 'Y': return 2u | 8u;
    case 'S': return 2u | 4u;
    case 'W': return 1u | 8u;
    case 'K': return 4u | 8u;
    case 'M': return 1u | 2u;
    case 'B': return 2u | 4u | 8u;
    case 'D': return 1u | 4u | 8u;
    case 'H': return 1u | 2u | 8u;
    case 'V': return 1u | 2u | 4u;
    case 'N': case '?': case '-': case '.': case 'O': case 'X': return 15u;
    default: return 0u;
  }
}

// Protein, bit i = amino acid i in the order A R N D C Q E G H I L K M F P S
// T W Y V; B = N|D, Z = Q|E, J = I|L; X ? - . * are every state.
uint32_t protein_mask(char ch) {
  static const char kOrder[] = "ARNDCQEGHILKMFPSTWYV";
  const char c = ch >= 'a' && ch <= 'z' ? (char)(ch - 32) : ch;
  for (int i = 0; i < 20; ++i)
    if (kOrder[i] == c) return 1u << i;
  switch (c) {
    case 'B': return (1u << 2) | (1u << 3);
    case 'Z': return (1u << 5) | (1u << 6);
    case 'J': return (1u << 9) | (1u << 10);
    case 'X': case '?': case '-': case '.': case '*': return (1u << 20) - 1u;
    default: return 0u;
  }
}

}  // namespace

extern "C" {

int netlk_encode_states(const char *chars, int64_t n, int32_t states, uint32_t *out_masks, int64_t *bad_index) {
  if (bad_index) *bad_index = -1;
  if ((!chars && n) || (!out_masks && n) || n < 0 || (states != 4 && states != 20)) {
    netlk::set_global_error("encode: characters, output and states 4 or 20 required");
    return NETLK_ERR_INVALID_ARGUMENT;
  }
  for (int64_t i = 0; i < n; ++i) {
    const uint32_t m = states == 4 ? dna_mask(chars[i]) : protein_mask(chars[i]);
    if (!m) {
      if (bad_index) *bad_index = i;
      netlk::set_global_error(std::string("encode: unknown character '") + chars[i] + "' at " + std::to_string(i));
      return NETLK_ERR_INVALID_ARGUMENT;
    }
    out_masks[i] = m;
  }
  return NETLK_OK;
}

int netlk_compress_patterns(const uint32_t *tip_states, int32_t n_tips, int64_t n_sites, uint32_t *out_patterns,
                            double *out_weights, int64_t *n_patterns) {
  if (!tip_states || !out_patterns || !out_weights || !n_patterns || n_tips <= 0 || n_sites < 0) {
    netlk::set_global_error("compress: arrays, n_tips > 0 and n_sites >= 0 required");
    return NETLK_ERR_INVALID_ARGUMENT;
  }
  // distinct columns in order of first occurrence
  struct Hash {
    size_t operator()(const std::string &s) const { return std::hash<std::string>()(s); }
  };
  std::unordered_map<std::string, int64_t, Hash> index;
  index.reserve((size_t)n_sites);
  std::vector<int64_t> first;
  std::vector<double> count;
  std::string key((size_t)n_tips * 4, '\0');
  for (int64_t s = 0; s < n_sites; ++s) {
    for (int32_t t = 0; t < n_tips; ++t) {
      const uint32_t v = tip_states[(size_t)t * n_sites + s];
      std::memcpy(&key[(size_t)t * 4], &v, 4);
    }
    auto it = index.find(key);
    if (it == index.end()) {
      index.emplace(key, (int64_t)first.size());
      first.push_back(s);
      count.push_back(1.0);
    } else {
      count[it->second] += 1.0;
    }
  }
  const int64_t np = (int64_t)first.size();
  for (int32_t t = 0; t < n_tips; ++t)
    for (int64_t j = 0; j < np; ++j) out_patterns[(size_t)t * np + j] = tip_states[(size_t)t * n_sites + first[j]];
  for (int64_t j = 0; j < np; ++j) out_weights[j] = count[j];
  *n_patterns = np;
  return NETLK_OK;
}

}  // extern "C"
