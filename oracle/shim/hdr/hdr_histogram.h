// Stand-in declarations for HdrHistogram_c (absent from this image).  The
// reference headers the oracle's drivers include mention these, but no
// driver calls them; the declarations just have to parse.
#pragma once
#include <cstdint>
#include <cstdio>
struct hdr_histogram {
  int64_t unused;
};
enum format_type { CLASSIC, CSV };
inline int hdr_percentiles_print(hdr_histogram*, FILE*, int, double, format_type) {
  return 0;
}
inline int hdr_init(int64_t, int64_t, int, hdr_histogram**) { return 0; }
inline bool hdr_record_value(hdr_histogram*, int64_t) { return true; }
inline void hdr_reset(hdr_histogram*) {}
inline void hdr_close(hdr_histogram*) {}
