// Checkpoint record of the reference (io.f90:1314-1338 `checkpoint`, read
// back by initial.f90:54-114 and :128-160) as one Fortran unformatted
// sequential record, and the record layer on its own.
//
// Record layout (the unformatted sequential format of gfortran and Intel
// Fortran, 4-byte markers): a logical record is one or more subrecords,
// each a leading 4-byte marker, at most 2147483639 data bytes and a trailing
// marker; a marker holds the subrecord's data length, negated in a leading
// marker when another subrecord follows and in a trailing marker when one
// precedes.  Markers and data are little-endian (the reference's x86 build
// writes them so; hosts of another byte order are refused).  Host code only.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "les_internal.h"

namespace {

constexpr long long kMaxSub = 2147483639LL;

bool little_endian() {
  const uint16_t x = 1;
  unsigned char b;
  std::memcpy(&b, &x, 1);
  return b == 1;
}
void put_marker(unsigned char* p, int32_t v) {
  const uint32_t u = (uint32_t)v;
  for (int i = 0; i < 4; ++i) p[i] = (unsigned char)(u >> (8 * i));
}
int32_t get_marker(const unsigned char* p) {
  uint32_t u = 0;
  for (int i = 0; i < 4; ++i) u |= (uint32_t)p[i] << (8 * i);
  return (int32_t)u;
}

// Writes one logical record of known total length, splitting it into
// subrecords of at most max_sub bytes.
class RecordWriter {
 public:
  RecordWriter(FILE* fp, long long total, long long max_sub) : fp_(fp), total_(total), max_(max_sub) {
    open_sub();
  }
  bool write(const void* data, long long n) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    if (done_ + n > total_) ok_ = false;  // more bytes than the record was opened for
    while (n > 0 && ok_) {
      if (cur_done_ == cur_len_) {  // current subrecord full: close it, open the next
        close_sub();
        ++sub_;
        open_sub();
      }
      const long long k = std::min(n, cur_len_ - cur_done_);
      if (fwrite(p, 1, (size_t)k, fp_) != (size_t)k) ok_ = false;
      p += k; n -= k; cur_done_ += k; done_ += k;
    }
    return ok_;
  }
  bool finish() {
    if (done_ != total_) ok_ = false;
    if (ok_) close_sub();
    return ok_;
  }

 private:
  void open_sub() {
    cur_len_ = std::min(max_, total_ - done_);
    cur_done_ = 0;
    unsigned char m[4];
    put_marker(m, (int32_t)(total_ - done_ > cur_len_ ? -cur_len_ : cur_len_));
    if (fwrite(m, 1, 4, fp_) != 4) ok_ = false;
  }
  void close_sub() {
    unsigned char m[4];
    put_marker(m, (int32_t)(sub_ > 0 ? -cur_len_ : cur_len_));
    if (fwrite(m, 1, 4, fp_) != 4) ok_ = false;
  }
  FILE* fp_;
  long long total_, max_, done_ = 0, cur_len_ = 0, cur_done_ = 0;
  int sub_ = 0;
  bool ok_ = true;
};

// Reads one logical record front to back; read() may stop short of the
// record's end, skip_rest() consumes what is left.
class RecordReader {
 public:
  explicit RecordReader(FILE* fp) : fp_(fp) { open_sub(); }
  bool read(void* dst, long long n) {
    unsigned char* p = static_cast<unsigned char*>(dst);
    while (n > 0 && ok_) {
      if (left_ == 0 && !next_sub()) {
        if (ok_) fail("the record holds fewer bytes than the list needs");
        return false;
      }
      const long long k = std::min(n, left_);
      if (fread(p, 1, (size_t)k, fp_) != (size_t)k) { fail("file ends inside a record"); return false; }
      p += k; n -= k; left_ -= k; got_ += k;
    }
    return ok_;
  }
  bool skip_rest() {
    while (ok_) {
      if (left_ > 0) {
        if (fseeko(fp_, (off_t)left_, SEEK_CUR) != 0) { fail("file ends inside a record"); break; }
        got_ += left_;
        left_ = 0;
      }
      if (!next_sub()) break;
    }
    return ok_;
  }
  long long record_bytes() const { return got_; }
  bool ok() const { return ok_; }
  const char* why() const { return why_; }

 private:
  void fail(const char* w) { ok_ = false; why_ = w; }
  void open_sub() {
    unsigned char m[4];
    if (fread(m, 1, 4, fp_) != 4) { fail("no record at this offset"); return; }
    const int32_t h = get_marker(m);
    more_ = h < 0;
    len_ = h < 0 ? -(long long)h : (long long)h;
    left_ = len_;
  }
  // close the current subrecord (its trailing marker must match) and open
  // the next one; false at the end of the record
  bool next_sub() {
    unsigned char m[4];
    if (fread(m, 1, 4, fp_) != 4) { fail("file ends inside a record"); return false; }
    const int32_t t = get_marker(m);
    const long long tl = t < 0 ? -(long long)t : (long long)t;
    if (tl != len_ || (t < 0) != (sub_ > 0)) { fail("record markers do not match"); return false; }
    if (!more_) return false;
    ++sub_;
    open_sub();
    if (ok_ && sub_ > 0 && len_ == 0 && more_) { fail("empty continued subrecord"); return false; }
    return ok_;
  }
  FILE* fp_;
  long long len_ = 0, left_ = 0, got_ = 0;
  int sub_ = 0;
  bool more_ = false, ok_ = true;
  const char* why_ = "";
};

// Items of the checkpoint record in order (io.f90:1325-1335).
enum ItemKind { VOL, VOL_ZERO, VOL_PR, SFC_LD, SFC_LD_ZERO, PLANE };
struct Item {
  ItemKind kind;
  int field;  // LES_* for VOL, SFC_LD, PLANE
};
// Without humidity (q_flag = 0) qmix, RHS_q and sgs_q3 are written as the
// zeros a run of the reference holds for them and skipped on reading; outside
// model 7 G_LM..G_NN likewise, and Pr_t as the constant Pr.
std::vector<Item> record_items(const les_ctx* c) {
  const bool q = c->cfg.q_flag != 0;
  const bool m7 = c->cfg.model == 7;
  const Item qv = q ? Item{VOL, LES_Q} : Item{VOL_ZERO, -1};
  const Item qr = q ? Item{VOL, LES_RHS_Q} : Item{VOL_ZERO, -1};
  const Item q3 = q ? Item{SFC_LD, LES_SGS_Q3_SFC} : Item{SFC_LD_ZERO, -1};
  auto g7 = [&](int f) { return m7 ? Item{VOL, f} : Item{VOL_ZERO, -1}; };
  if (c->cfg.s_flag)
    return {{VOL, LES_U},       {VOL, LES_V},       {VOL, LES_W},       {VOL, LES_THETA},   qv,  // qmix
            {VOL, LES_RHSX},    {VOL, LES_RHSY},    {VOL, LES_RHSZ},    {VOL, LES_RHS_T},   qr,  // RHS_q
            {SFC_LD, LES_SGS_T3_SFC}, q3,                                                        // sgs_t3, sgs_q3
            {PLANE, LES_PSI_M}, {PLANE, LES_PSI_M0}, {PLANE, LES_PSI_H}, {PLANE, LES_PSI_H0},
            {VOL, LES_CS_OPT2}, {VOL, LES_F_LM},    {VOL, LES_F_MM},    {VOL, LES_F_QN},    {VOL, LES_F_NN},
            g7(LES_G_LM),       g7(LES_G_MM),       g7(LES_G_QN),       g7(LES_G_NN),
            m7 ? Item{VOL, LES_PR_T} : Item{VOL_PR, -1}};
  return {{VOL, LES_U},    {VOL, LES_V},       {VOL, LES_W},    {VOL, LES_RHSX},
          {VOL, LES_RHSY}, {VOL, LES_RHSZ},    {VOL, LES_CS_OPT2}, {VOL, LES_F_LM},
          {VOL, LES_F_MM}, {VOL, LES_F_QN},    {VOL, LES_F_NN}};
}
size_t item_elems(const les_ctx* c, const Item& it) {
  const les::Grid& g = c->g;
  switch (it.kind) {
    case VOL: case VOL_ZERO: case VOL_PR: return (size_t)g.ld * g.ny * g.nz;
    case SFC_LD: case SFC_LD_ZERO: return (size_t)g.ld * g.ny;
    default: return (size_t)g.nx * g.ny;
  }
}

}  // namespace

extern "C" {

int les_fortran_record_write(const char* path, int append, const void* const* parts, const size_t* nbytes,
                             int nparts, long long max_subrecord) {
  if (!path || nparts < 0 || (nparts > 0 && (!parts || !nbytes))) return LES_ERR_ARG;
  if (!little_endian()) { les_set_error("record files are little-endian; this host is not"); return LES_ERR_UNSUPPORTED; }
  const long long maxs = max_subrecord > 0 ? std::min(max_subrecord, kMaxSub) : kMaxSub;
  long long total = 0;
  for (int i = 0; i < nparts; ++i) {
    if (nbytes[i] > 0 && !parts[i]) return LES_ERR_ARG;
    total += (long long)nbytes[i];
  }
  FILE* fp = fopen(path, append ? "ab" : "wb");
  if (!fp) { les_set_error("cannot open %s for writing", path); return LES_ERR_IO; }
  RecordWriter w(fp, total, maxs);
  bool ok = true;
  for (int i = 0; i < nparts && ok; ++i) ok = w.write(parts[i], (long long)nbytes[i]);
  ok = ok && w.finish();
  ok = (fclose(fp) == 0) && ok;
  if (!ok) { les_set_error("write to %s failed", path); return LES_ERR_IO; }
  return LES_OK;
}

int les_fortran_record_read(const char* path, long long offset, void* const* parts, const size_t* nbytes, int nparts,
                            long long* record_bytes, long long* next_offset) {
  if (!path || offset < 0 || nparts < 0 || (nparts > 0 && (!parts || !nbytes))) return LES_ERR_ARG;
  if (!little_endian()) { les_set_error("record files are little-endian; this host is not"); return LES_ERR_UNSUPPORTED; }
  FILE* fp = fopen(path, "rb");
  if (!fp) { les_set_error("cannot open %s for reading", path); return LES_ERR_IO; }
  if (fseeko(fp, (off_t)offset, SEEK_SET) != 0) { fclose(fp); les_set_error("cannot seek in %s", path); return LES_ERR_IO; }
  RecordReader r(fp);
  for (int i = 0; i < nparts && r.ok(); ++i)
    if (nbytes[i] > 0 && !r.read(parts[i], (long long)nbytes[i])) break;
  if (r.ok()) r.skip_rest();
  const long long pos = (long long)ftello(fp);
  fclose(fp);
  if (!r.ok()) { les_set_error("%s at offset %lld: %s", path, offset, r.why()); return LES_ERR_IO; }
  if (record_bytes) *record_bytes = r.record_bytes();
  if (next_offset) *next_offset = pos;
  return LES_OK;
}

int les_checkpoint_write(les_ctx* c, const char* path) {
  if (!c || !path) return LES_ERR_ARG;
  if (!little_endian()) { les_set_error("record files are little-endian; this host is not"); return LES_ERR_UNSUPPORTED; }
  const les::Grid& g = c->g;
  const std::vector<Item> items = record_items(c);
  long long total = 0;
  for (const Item& it : items) total += (long long)item_elems(c, it) * 8;
  std::vector<double> buf((size_t)g.ld * g.ny * g.nz), sfc((size_t)g.nx * g.ny);
  FILE* fp = fopen(path, "wb");
  if (!fp) { les_set_error("cannot open %s for writing", path); return LES_ERR_IO; }
  RecordWriter w(fp, total, kMaxSub);
  int st = LES_OK;
  for (const Item& it : items) {
    const size_t n = item_elems(c, it);
    switch (it.kind) {
      case VOL: case PLANE: st = les_get_field(c, (les_field)it.field, buf.data()); break;
      case VOL_ZERO: case SFC_LD_ZERO: std::fill(buf.begin(), buf.begin() + n, 0.0); break;
      case VOL_PR: std::fill(buf.begin(), buf.begin() + n, c->cfg.pr); break;  // sgs_stag.f90:171 Pr_t = Pr
      case SFC_LD:  // (nx,ny) surface flux into the (ld,ny) plane sgs_t3(:,:,1), padding columns 0
        st = les_get_field(c, (les_field)it.field, sfc.data());
        std::fill(buf.begin(), buf.begin() + n, 0.0);
        for (int jy = 0; jy < g.ny; ++jy)
          std::memcpy(&buf[(size_t)jy * g.ld], &sfc[(size_t)jy * g.nx], (size_t)g.nx * sizeof(double));
        break;
    }
    if (st != LES_OK) break;
    if (!w.write(buf.data(), (long long)n * 8)) { st = LES_ERR_IO; break; }
  }
  if (st == LES_OK && !w.finish()) st = LES_ERR_IO;
  if (fclose(fp) != 0 && st == LES_OK) st = LES_ERR_IO;
  if (st == LES_ERR_IO) les_set_error("write to %s failed", path);
  return st;
}

int les_checkpoint_read(les_ctx* c, const char* path) {
  if (!c || !path) return LES_ERR_ARG;
  if (!little_endian()) { les_set_error("record files are little-endian; this host is not"); return LES_ERR_UNSUPPORTED; }
  const les::Grid& g = c->g;
  const std::vector<Item> items = record_items(c);
  // the record must hold exactly this configuration's list (a record written
  // with scalars does not read into a context without them, nor the other
  // way round); checked before any field changes
  long long total = 0, rec = 0;
  for (const Item& it : items) total += (long long)item_elems(c, it) * 8;
  if (int st0 = les_fortran_record_read(path, 0, nullptr, nullptr, 0, &rec, nullptr)) return st0;
  if (rec != total) {
    les_set_error("%s: the record holds %lld bytes, the checkpoint list of this configuration %lld", path, rec,
                  total);
    return LES_ERR_IO;
  }
  std::vector<double> buf((size_t)g.ld * g.ny * g.nz), sfc((size_t)g.nx * g.ny);
  FILE* fp = fopen(path, "rb");
  if (!fp) { les_set_error("cannot open %s for reading", path); return LES_ERR_IO; }
  RecordReader r(fp);
  int st = LES_OK;
  for (const Item& it : items) {
    const size_t n = item_elems(c, it);
    if (!r.read(buf.data(), (long long)n * 8)) break;
    switch (it.kind) {
      case VOL: case PLANE: st = les_set_field(c, (les_field)it.field, buf.data()); break;
      case SFC_LD:
        for (int jy = 0; jy < g.ny; ++jy)
          std::memcpy(&sfc[(size_t)jy * g.nx], &buf[(size_t)jy * g.ld], (size_t)g.nx * sizeof(double));
        st = les_set_field(c, (les_field)it.field, sfc.data());
        break;
      default: break;  // the zero and constant items of this configuration
    }
    if (st != LES_OK) break;
  }
  if (st == LES_OK && r.ok()) r.skip_rest();
  fclose(fp);
  if (st == LES_OK && !r.ok()) {
    les_set_error("%s: %s", path, r.why());
    st = LES_ERR_IO;
  }
  return st;
}

}  // extern "C"
