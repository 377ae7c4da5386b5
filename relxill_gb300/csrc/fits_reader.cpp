// fits_reader.cpp -- see fits_reader.h
#include "fits_reader.h"

#include <cctype>
#include <cstdlib>
#include <cstring>

namespace relx {

static constexpr int64_t kBlock = 2880;

float be_f32(const unsigned char *p) {
  uint32_t u = ((uint32_t) p[0] << 24) | ((uint32_t) p[1] << 16) | ((uint32_t) p[2] << 8) | p[3];
  float v;
  std::memcpy(&v, &u, 4);
  return v;
}
double be_f64(const unsigned char *p) {
  uint64_t u = 0;
  for (int i = 0; i < 8; i++) u = (u << 8) | p[i];
  double v;
  std::memcpy(&v, &u, 8);
  return v;
}
int32_t be_i32(const unsigned char *p) {
  uint32_t u = ((uint32_t) p[0] << 24) | ((uint32_t) p[1] << 16) | ((uint32_t) p[2] << 8) | p[3];
  return (int32_t) u;
}
static int elem_size(char c) {
  switch (c) {
    case 'E': case 'J': return 4;
    case 'D': case 'K': return 8;
    case 'I': return 2;
    case 'A': case 'B': case 'L': return 1;
    default: return 0;
  }
}
static std::string lower(std::string s) {
  for (auto &ch : s) ch = (char) std::tolower((unsigned char) ch);
  return s;
}
static std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(' '), b = s.find_last_not_of(' ');
  if (a == std::string::npos) return "";
  return s.substr(a, b - a + 1);
}
static std::string card_value(const char *card) {
  std::string v(card + 10, 70);
  size_t p = v.find_first_not_of(' ');
  if (p == std::string::npos) return "";
  if (v[p] == '\'') {
    std::string out;
    for (size_t i = p + 1; i < v.size(); i++) {
      if (v[i] == '\'') {
        if (i + 1 < v.size() && v[i + 1] == '\'') { out += '\''; i++; continue; }
        break;
      }
      out += v[i];
    }
    return trim(out);
  }
  size_t slash = v.find('/');
  if (slash != std::string::npos) v = v.substr(0, slash);
  return trim(v);
}

int FitsHdu::col(const std::string &name) const {
  std::string n = lower(name);
  for (size_t i = 0; i < cols.size(); i++)
    if (lower(cols[i].name) == n) return (int) i;
  return -1;
}

FitsFile::~FitsFile() {
  if (fp_) std::fclose(fp_);
}

bool FitsFile::open(const std::string &path, std::string *err) {
  fp_ = std::fopen(path.c_str(), "rb");
  if (!fp_) {
    if (err) *err = "cannot open " + path;
    return false;
  }
  int64_t pos = 0;
  std::vector<char> block(kBlock);
  while (true) {
    if (fseeko(fp_, pos, SEEK_SET) != 0) break;
    FitsHdu h;
    int64_t naxis = 0, naxis1 = 0, naxis2 = 0, pcount = 0, tfields = 0;
    bool bintable = false, ended = false;
    int64_t nbytes = 0;
    std::vector<std::string> ttype, tform;
    while (!ended) {
      if ((int64_t) std::fread(block.data(), 1, kBlock, fp_) != kBlock) {
        if (hdus_.empty() && err) *err = "not a FITS file: " + path;
        return !hdus_.empty();
      }
      nbytes += kBlock;
      for (int i = 0; i < kBlock; i += 80) {
        const char *card = block.data() + i;
        std::string key = trim(std::string(card, 8));
        if (key == "END") { ended = true; break; }
        if (card[8] != '=') continue;
        std::string val = card_value(card);
        if (key == "XTENSION") bintable = (val == "BINTABLE");
        else if (key == "NAXIS") naxis = std::atoll(val.c_str());
        else if (key == "NAXIS1") naxis1 = std::atoll(val.c_str());
        else if (key == "NAXIS2") naxis2 = std::atoll(val.c_str());
        else if (key == "PCOUNT") pcount = std::atoll(val.c_str());
        else if (key == "TFIELDS") {
          tfields = std::atoll(val.c_str());
          ttype.assign(tfields + 1, "");
          tform.assign(tfields + 1, "");
        } else if (key == "EXTNAME") h.extname = val;
        else if (key.compare(0, 5, "TTYPE") == 0) {
          int k = std::atoi(key.c_str() + 5);
          if (k >= 1 && k <= tfields) ttype[k] = val;
        } else if (key.compare(0, 5, "TFORM") == 0) {
          int k = std::atoi(key.c_str() + 5);
          if (k >= 1 && k <= tfields) tform[k] = val;
        }
      }
    }
    h.data_off = pos + nbytes;
    int64_t datasize = 0;
    if (bintable && naxis == 2) {
      h.is_table = true;
      h.width = naxis1;
      h.nrows = naxis2;
      int64_t off = 0;
      for (int k = 1; k <= tfields; k++) {
        FitsColumn c;
        c.name = ttype[k];
        const std::string &tf = tform[k];
        size_t j = 0;
        while (j < tf.size() && std::isdigit((unsigned char) tf[j])) j++;
        c.repeat = j ? std::atoll(tf.substr(0, j).c_str()) : 1;
        c.code = j < tf.size() ? tf[j] : 'E';
        c.offset = off;
        off += c.repeat * elem_size(c.code);
        h.cols.push_back(c);
      }
      datasize = naxis1 * naxis2 + pcount;
    }
    hdus_.push_back(h);
    pos = h.data_off + ((datasize + kBlock - 1) / kBlock) * kBlock;
  }
  return true;
}

const FitsHdu *FitsFile::find(const std::string &extname) const {
  std::string n = lower(extname);
  for (auto &h : hdus_)
    if (lower(h.extname) == n) return &h;
  return nullptr;
}

bool FitsFile::read_rows(const FitsHdu &h, int64_t r0, int64_t nr, unsigned char *out) const {
  if (r0 < 0 || r0 + nr > h.nrows) return false;
  if (fseeko(fp_, h.data_off + r0 * h.width, SEEK_SET) != 0) return false;
  return (int64_t) std::fread(out, 1, (size_t) (nr * h.width), fp_) == nr * h.width;
}

template <typename T>
static bool read_num(const FitsFile &f, const FitsHdu &h, int c, int64_t r0, int64_t nr, T *out) {
  if (c < 0 || c >= (int) h.cols.size()) return false;
  const FitsColumn &col = h.cols[c];
  std::vector<unsigned char> buf((size_t) (nr * h.width));
  if (!f.read_rows(h, r0, nr, buf.data())) return false;
  const int es = elem_size(col.code);
  for (int64_t r = 0; r < nr; r++) {
    const unsigned char *p = buf.data() + r * h.width + col.offset;
    for (int64_t e = 0; e < col.repeat; e++, p += es) {
      double v;
      switch (col.code) {
        case 'E': v = be_f32(p); break;
        case 'D': v = be_f64(p); break;
        case 'J': v = be_i32(p); break;
        case 'I': v = (int16_t) (((uint16_t) p[0] << 8) | p[1]); break;
        default: return false;
      }
      out[r * col.repeat + e] = (T) v;
    }
  }
  return true;
}

bool FitsFile::read_f64(const FitsHdu &h, int c, int64_t r0, int64_t nr, double *out) const {
  return read_num<double>(*this, h, c, r0, nr, out);
}
bool FitsFile::read_f32(const FitsHdu &h, int c, int64_t r0, int64_t nr, float *out) const {
  if (c >= 0 && c < (int) h.cols.size() && h.cols[c].code == 'E') {
    // exact float copy without a double round trip
    const FitsColumn &col = h.cols[c];
    std::vector<unsigned char> buf((size_t) (nr * h.width));
    if (!read_rows(h, r0, nr, buf.data())) return false;
    for (int64_t r = 0; r < nr; r++) {
      const unsigned char *p = buf.data() + r * h.width + col.offset;
      for (int64_t e = 0; e < col.repeat; e++) out[r * col.repeat + e] = be_f32(p + 4 * e);
    }
    return true;
  }
  return read_num<float>(*this, h, c, r0, nr, out);
}
bool decode_f32(const FitsHdu &h, int c, const unsigned char *rows, int64_t nr, float *out) {
  if (c < 0 || c >= (int) h.cols.size() || h.cols[c].code != 'E') return false;
  const FitsColumn &col = h.cols[c];
  for (int64_t r = 0; r < nr; r++) {
    const unsigned char *p = rows + r * h.width + col.offset;
    for (int64_t e = 0; e < col.repeat; e++) out[r * col.repeat + e] = be_f32(p + 4 * e);
  }
  return true;
}

bool FitsFile::read_str(const FitsHdu &h, int c, int64_t r0, int64_t nr, std::vector<std::string> *out) const {
  if (c < 0 || c >= (int) h.cols.size() || h.cols[c].code != 'A') return false;
  const FitsColumn &col = h.cols[c];
  std::vector<unsigned char> buf((size_t) (nr * h.width));
  if (!read_rows(h, r0, nr, buf.data())) return false;
  out->clear();
  for (int64_t r = 0; r < nr; r++) {
    std::string s((const char *) buf.data() + r * h.width + col.offset, (size_t) col.repeat);
    size_t z = s.find('\0');
    if (z != std::string::npos) s.resize(z);
    out->push_back(trim(s));
  }
  return true;
}

}  // namespace relx
