// fits_reader.h -- read-only access to FITS binary tables (FITS standard
// v4.0, sections 4 and 7.3): HDU scan, column lookup by name, and reading of
// E/D/J/I/K/A columns as host arrays.  Enough for the relxill tables.
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace relx {

struct FitsColumn {
  std::string name;
  char code = 0;          // E, D, J, I, K, A, B
  int64_t repeat = 1;
  int64_t offset = 0;     // byte offset inside a row
};

struct FitsHdu {
  std::string extname;
  bool is_table = false;
  int64_t data_off = 0, width = 0, nrows = 0;
  std::vector<FitsColumn> cols;
  int col(const std::string &name) const;  // -1 if absent (case insensitive)
};

class FitsFile {
 public:
  bool open(const std::string &path, std::string *err);
  ~FitsFile();
  const std::vector<FitsHdu> &hdus() const { return hdus_; }
  const FitsHdu *find(const std::string &extname) const;
  // read column `c` of rows [r0, r0+nr) as doubles / floats (row-major, repeat values per row)
  bool read_f64(const FitsHdu &h, int c, int64_t r0, int64_t nr, double *out) const;
  bool read_f32(const FitsHdu &h, int c, int64_t r0, int64_t nr, float *out) const;
  bool read_str(const FitsHdu &h, int c, int64_t r0, int64_t nr, std::vector<std::string> *out) const;
  // raw big-endian bytes of rows [r0, r0+nr)
  bool read_rows(const FitsHdu &h, int64_t r0, int64_t nr, unsigned char *out) const;

 private:
  FILE *fp_ = nullptr;
  std::vector<FitsHdu> hdus_;
};

// decode float column `c` from raw rows already in memory (nr rows of h.width bytes)
bool decode_f32(const FitsHdu &h, int c, const unsigned char *rows, int64_t nr, float *out);

float be_f32(const unsigned char *p);
double be_f64(const unsigned char *p);
int32_t be_i32(const unsigned char *p);

}  // namespace relx
