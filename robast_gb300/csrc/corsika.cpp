// corsika.cpp -- reader of CORSIKA IACT photon-bunch files (the eventio
// stream that ACorsikaIACTFile reads, src/ACorsikaIACTFile.cxx:191-489),
// from an in-memory, already decompressed byte stream.
//
// eventio layout: a top-level block is a little-endian sync word
// 0xD41F8A37 followed by an item header; an item header is
//   u32 type/version (type = bits 0-15, version = bits 20-31),
//   i32 ident,
//   u32 length (bits 0-29; bit 30: the item holds only sub-items; bit 31:
//       an extension word follows whose bits 0-11 are length bits 30-41),
// then `length` bytes of data, which may contain sub-items with the same
// header minus the sync word.  Records used here (type numbers are those
// of CORSIKA's IACT option):
//   1200 run header, 1202 event header: i32 count, i32 first word, then
//        count-1 float32 (273 in all);
//   1212 input card: i32 line count, each line i16 length + bytes;
//   1201 telescope positions: i32 n, float32 x[n], y[n], z[n], r[n] (cm);
//   1203 array offsets: i32 n, float32 time offset, x[n], y[n] (version 1
//        adds weights[n]);
//   1204 telescope array (ident = array number) holding 1205 sub-items,
//        or 1213 array head, top-level 1205 blocks, 1214 array end;
//   1205 photon bunches: i16 array, i16 telescope, float32 photons,
//        i32 bunch count, then per bunch either 8 float32 (version 0: x, y,
//        cx, cy, time, zem, photons, lambda) or 8 int16 (version 1000:
//        0.1 x, 0.1 y, cx/30000, cy/30000, 0.1 time, 10^(0.001 zem),
//        0.01 photons, lambda);
//   1209 event end, 1210 run end.
// Every read is bounds-checked against its enclosing item: a malformed
// stream gives RBG_ERR_ARG, never an out-of-range access.
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "robast_gb.h"

struct rbg_corsika {
  std::vector<uint8_t> data;
  size_t pos = 0;  // next top-level block
  float runh[273] = {0};
  float evth[273] = {0};
  bool have_event = false;
  std::vector<std::string> input_lines;
  std::vector<double> tel_x, tel_y, tel_z, tel_r;
  int32_t n_arrays = 0;
  double time_offset = 0;
  std::vector<double> off_x, off_y;
  // bunches of the current event (structure of arrays)
  std::vector<int32_t> b_tel, b_array;
  std::vector<float> b_x, b_y, b_zem, b_time, b_cx, b_cy, b_cz, b_lambda, b_photons;
};

namespace {

constexpr uint32_t kSync = 0xD41F8A37u;
enum : int {
  kRunH = 1200,
  kTelPos = 1201,
  kEvtH = 1202,
  kTelOff = 1203,
  kTelArray = 1204,
  kPhotons = 1205,
  kEvtE = 1209,
  kRunE = 1210,
  kInputCfg = 1212,
  kTelArrayHead = 1213,
  kTelArrayEnd = 1214
};

struct Cursor {
  const uint8_t* p;
  size_t n, i;
  bool ok = true;
  bool need(size_t k) {
    if (!ok || i + k > n) ok = false;
    return ok;
  }
  uint32_t u32() {
    if (!need(4)) return 0;
    uint32_t v = (uint32_t)p[i] | ((uint32_t)p[i + 1] << 8) | ((uint32_t)p[i + 2] << 16) | ((uint32_t)p[i + 3] << 24);
    i += 4;
    return v;
  }
  int32_t i32() { return (int32_t)u32(); }
  int16_t i16() {
    if (!need(2)) return 0;
    uint16_t v = (uint16_t)(p[i] | (p[i + 1] << 8));
    i += 2;
    return (int16_t)v;
  }
  float f32() {
    uint32_t u = u32();
    float f;
    std::memcpy(&f, &u, 4);
    return f;
  }
};

struct Item {
  int type = 0, version = 0;
  int32_t ident = 0;
  size_t begin = 0, end = 0;  // data range
};

// header at c.i (no sync word); the item's data must fit in [c.i, limit)
bool read_header(Cursor& c, size_t limit, Item& it) {
  const uint32_t tv = c.u32();
  it.ident = c.i32();
  uint64_t len = c.u32();
  if (!c.ok) return false;
  it.type = (int)(tv & 0xffffu);
  it.version = (int)((tv >> 20) & 0xfffu);
  if (len & 0x80000000u) {
    const uint32_t ext = c.u32();
    if (!c.ok) return false;
    len = (len & 0x3fffffffu) | ((uint64_t)(ext & 0xfffu) << 30);
  } else {
    len &= 0x3fffffffu;
  }
  it.begin = c.i;
  if (len > limit - c.i) return false;
  it.end = c.i + (size_t)len;
  return true;
}

// next top-level block: sync word + header; false at the end of the stream
bool next_block(rbg_corsika* f, Item& it, bool& bad) {
  bad = false;
  if (f->pos >= f->data.size()) return false;
  Cursor c{f->data.data(), f->data.size(), f->pos};
  if (c.u32() != kSync || !c.ok) {
    bad = true;
    return false;
  }
  if (!read_header(c, f->data.size(), it)) {
    bad = true;
    return false;
  }
  f->pos = it.end;
  return true;
}

bool read_header_block(const rbg_corsika* f, const Item& it, float* out) {
  if (it.version != 0) return false;
  Cursor c{f->data.data(), it.end, it.begin};
  const int32_t len = c.i32();
  if (!c.ok || len < 1 || len > 273) return false;
  const int32_t first = c.i32();
  std::memcpy(&out[0], &first, 4);
  for (int k = 1; k < len; ++k) out[k] = c.f32();
  for (int k = len; k < 273; ++k) out[k] = 0.f;
  return c.ok;
}

// one photons item (1205) at [it.begin, it.end)
bool read_photons(rbg_corsika* f, const Item& it) {
  const int fmt = it.version / 1000;
  if (it.version % 1000 != 0 || fmt > 1) return false;
  Cursor c{f->data.data(), it.end, it.begin};
  const int32_t array = c.i16(), tel = c.i16();
  (void)c.f32();  // sum of photons in this device
  const int32_t nb = c.i32();
  if (!c.ok || nb < 0) return false;
  const size_t per = fmt == 0 ? 32 : 16;
  if ((size_t)nb * per > it.end - c.i) return false;
  for (int32_t j = 0; j < nb; ++j) {
    float x, y, cx, cy, t, zem, ph, lam;
    if (fmt == 0) {
      x = c.f32();
      y = c.f32();
      cx = c.f32();
      cy = c.f32();
      t = c.f32();
      zem = c.f32();
      ph = c.f32();
      lam = c.f32();
    } else {
      x = (float)(0.1 * c.i16());
      y = (float)(0.1 * c.i16());
      double v = c.i16() / 30000.;
      cx = (float)(v > 1. ? 1. : (v < -1. ? -1. : v));
      v = c.i16() / 30000.;
      cy = (float)(v > 1. ? 1. : (v < -1. ? -1. : v));
      t = (float)(0.1 * c.i16());
      zem = (float)std::pow(10., 0.001 * c.i16());
      ph = (float)(0.01 * c.i16());
      lam = (float)c.i16();
    }
    f->b_tel.push_back(tel);
    f->b_array.push_back(array);
    f->b_x.push_back(x);
    f->b_y.push_back(y);
    f->b_cx.push_back(cx);
    f->b_cy.push_back(cy);
    // ACorsikaIACTFile::ReadEvent (:450-452): cz = -sqrt(1 - cx^2 - cy^2)
    // with the squares taken in float
    const float cx2 = cx * cx, cy2 = cy * cy;
    f->b_cz.push_back((float)(-1. * std::sqrt(1. - cx2 - cy2)));
    f->b_time.push_back(t);
    f->b_zem.push_back(zem);
    f->b_lambda.push_back(lam);
    f->b_photons.push_back(ph);
  }
  return c.ok;
}

void clear_bunches(rbg_corsika* f) {
  for (auto* v : {&f->b_tel, &f->b_array}) v->clear();
  for (auto* v : {&f->b_x, &f->b_y, &f->b_zem, &f->b_time, &f->b_cx, &f->b_cy, &f->b_cz, &f->b_lambda, &f->b_photons})
    v->clear();
}

}  // namespace

extern "C" {

int rbg_corsika_open(const uint8_t* data, int64_t nbytes, rbg_corsika** out) {
  if (!data || nbytes <= 0 || !out) return RBG_ERR_ARG;
  *out = nullptr;
  rbg_corsika* f = new (std::nothrow) rbg_corsika();
  if (!f) return RBG_ERR_NOMEM;
  try {
    f->data.assign(data, data + nbytes);
  } catch (const std::bad_alloc&) {
    delete f;
    return RBG_ERR_NOMEM;
  }
  // ACorsikaIACTFile::Open (:191-257): run header, input card, positions
  const int order[3] = {kRunH, kInputCfg, kTelPos};
  for (int k = 0; k < 3; ++k) {
    Item it;
    bool bad;
    if (!next_block(f, it, bad) || it.type != order[k]) {
      delete f;
      return RBG_ERR_ARG;
    }
    bool ok = true;
    if (it.type == kRunH) {
      ok = read_header_block(f, it, f->runh);
    } else if (it.type == kInputCfg) {
      // lines: i16 length + bytes; empty lines are skipped, and a line
      // declared past the item's end ends the card (CORSIKA writers may
      // count one line more than they store; the reference's reader stops
      // there too)
      Cursor c{f->data.data(), it.end, it.begin};
      const int32_t n = c.i32();
      for (int32_t l = 0; c.ok && l < n && c.i + 2 <= it.end; ++l) {
        const int16_t len = c.i16();
        if (len <= 0) continue;
        if ((size_t)len > it.end - c.i) break;
        f->input_lines.emplace_back(reinterpret_cast<const char*>(c.p + c.i), (size_t)len);
        c.i += (size_t)len;
      }
      ok = it.version == 0;
    } else {
      Cursor c{f->data.data(), it.end, it.begin};
      const int32_t n = c.i32();
      ok = c.ok && it.version == 0 && n >= 0 && (size_t)n * 16 <= it.end - c.i;
      for (auto* v : {&f->tel_x, &f->tel_y, &f->tel_z, &f->tel_r})
        for (int32_t i = 0; ok && i < n; ++i) v->push_back(c.f32());
      ok = ok && c.ok;
    }
    if (!ok) {
      delete f;
      return RBG_ERR_ARG;
    }
  }
  *out = f;
  return RBG_OK;
}

void rbg_corsika_close(rbg_corsika* f) { delete f; }

int rbg_corsika_run_header(const rbg_corsika* f, float* out273) {
  if (!f || !out273) return RBG_ERR_ARG;
  std::memcpy(out273, f->runh, sizeof(f->runh));
  return RBG_OK;
}

int rbg_corsika_input_lines(const rbg_corsika* f, char* buf, int64_t cap, int32_t* n_lines) {
  if (!f) return RBG_ERR_ARG;
  if (n_lines) *n_lines = (int32_t)f->input_lines.size();
  std::string all;
  for (const auto& l : f->input_lines) all += l + "\n";
  if (buf && cap > 0) {
    const size_t k = all.size() < (size_t)cap - 1 ? all.size() : (size_t)cap - 1;
    std::memcpy(buf, all.data(), k);
    buf[k] = '\0';
  }
  return (int)all.size() + 1;
}

int rbg_corsika_telescopes(const rbg_corsika* f, int32_t cap, int32_t* n_tel, double* x, double* y, double* z,
                           double* r) {
  if (!f || !n_tel) return RBG_ERR_ARG;
  *n_tel = (int32_t)f->tel_x.size();
  for (int32_t i = 0; i < *n_tel && i < cap; ++i) {
    if (x) x[i] = f->tel_x[i];
    if (y) y[i] = f->tel_y[i];
    if (z) z[i] = f->tel_z[i];
    if (r) r[i] = f->tel_r[i];
  }
  return RBG_OK;
}

// ACorsikaIACTFile::ReadEvent (:264-489): read forward to the event with
// the given number (numbers start at 1) and keep its bunches.  An event
// is complete after its event header, array offsets, telescope arrays and
// event end.  *event = num, or -1 when the stream ends first (events cannot
// be read backwards, as in the reference); returns RBG_ERR_ARG on a
// malformed block, else RBG_OK.
int rbg_corsika_read_event(rbg_corsika* f, int32_t num, int32_t* event) {
  if (!f || !event) return RBG_ERR_ARG;
  *event = -1;
  if (f->have_event && (int32_t)f->evth[1] == num) {
    *event = num;
    return RBG_OK;
  }
  if (f->have_event && (int32_t)f->evth[1] > num) return RBG_OK;
  bool in_event = false, have_off = false, have_arrays = false, in_head = false;
  for (;;) {
    Item it;
    bool bad;
    if (!next_block(f, it, bad)) return bad ? RBG_ERR_ARG : RBG_OK;
    switch (it.type) {
      case kEvtH: {
        float h[273];
        if (!read_header_block(f, it, h)) return RBG_ERR_ARG;
        in_event = (int32_t)h[1] == num;
        have_off = have_arrays = false;
        if (in_event) {
          std::memcpy(f->evth, h, sizeof(h));
          f->have_event = true;
          clear_bunches(f);
        }
        break;
      }
      case kTelOff: {
        if (!in_event) break;
        if (it.version != 0 && it.version != 1) return RBG_ERR_ARG;
        Cursor c{f->data.data(), it.end, it.begin};
        const int32_t n = c.i32();
        f->time_offset = c.f32();
        if (!c.ok || n < 0 || (size_t)n * 8 > it.end - c.i) return RBG_ERR_ARG;
        f->n_arrays = n;
        f->off_x.assign(n, 0.0);
        f->off_y.assign(n, 0.0);
        for (int32_t i = 0; i < n; ++i) f->off_x[i] = c.f32();
        for (int32_t i = 0; i < n; ++i) f->off_y[i] = c.f32();
        if (!c.ok) return RBG_ERR_ARG;
        have_off = true;
        break;
      }
      case kTelArray: {
        if (!in_event || !have_off) break;
        if (it.version != 0) return RBG_ERR_ARG;
        Cursor c{f->data.data(), it.end, it.begin};
        while (c.ok && c.i + 12 <= it.end) {
          Item sub;
          if (!read_header(c, it.end, sub)) return RBG_ERR_ARG;
          if (sub.type == kPhotons && !read_photons(f, sub)) return RBG_ERR_ARG;
          c.i = sub.end;
        }
        have_arrays = true;
        break;
      }
      case kTelArrayHead:
        // per-telescope photon blocks follow at the top level
        in_head = in_event && have_off;
        if (in_head) have_arrays = true;
        break;
      case kPhotons:
        // a top-level photons block counts only inside an array head/end
        // pair (the reference ignores others, such as the summary block)
        if (in_head && !read_photons(f, it)) return RBG_ERR_ARG;
        break;
      case kTelArrayEnd:
        in_head = false;
        break;
      case kEvtE:
        if (in_event && have_off && have_arrays) {
          *event = num;
          return RBG_OK;
        }
        break;
      default:  // longitudinal profiles, extra parameters, run end, ...
        break;
    }
  }
}

int rbg_corsika_event_header(const rbg_corsika* f, float* out273) {
  if (!f || !out273 || !f->have_event) return RBG_ERR_ARG;
  std::memcpy(out273, f->evth, sizeof(f->evth));
  return RBG_OK;
}

int rbg_corsika_offsets(const rbg_corsika* f, int32_t cap, int32_t* n_arrays, double* time_offset, double* x,
                        double* y) {
  if (!f || !n_arrays || !f->have_event) return RBG_ERR_ARG;
  *n_arrays = f->n_arrays;
  if (time_offset) *time_offset = f->time_offset;
  for (int32_t i = 0; i < f->n_arrays && i < cap; ++i) {
    if (x) x[i] = f->off_x[i];
    if (y) y[i] = f->off_y[i];
  }
  return RBG_OK;
}

int64_t rbg_corsika_bunch_count(const rbg_corsika* f, int32_t tel, int32_t array) {
  if (!f) return RBG_ERR_ARG;
  int64_t n = 0;
  for (size_t i = 0; i < f->b_tel.size(); ++i)
    if ((tel < 0 || f->b_tel[i] == tel) && (array < 0 || f->b_array[i] == array)) ++n;
  return n;
}

// The bunches of telescope `tel` and array `array` (< 0: any) of the
// current event into host arrays of capacity out->n; out->n becomes the
// number written.  Any array pointer may be null.
int rbg_corsika_get_bunches(const rbg_corsika* f, int32_t tel, int32_t array, rbg_bunches* out) {
  if (!f || !out || out->n < 0) return RBG_ERR_ARG;
  int64_t k = 0;
  for (size_t i = 0; i < f->b_tel.size() && k < out->n; ++i) {
    if ((tel >= 0 && f->b_tel[i] != tel) || (array >= 0 && f->b_array[i] != array)) continue;
    if (out->tel) out->tel[k] = f->b_tel[i];
    if (out->array) out->array[k] = f->b_array[i];
    if (out->x) out->x[k] = f->b_x[i];
    if (out->y) out->y[k] = f->b_y[i];
    if (out->zem) out->zem[k] = f->b_zem[i];
    if (out->time) out->time[k] = f->b_time[i];
    if (out->cx) out->cx[k] = f->b_cx[i];
    if (out->cy) out->cy[k] = f->b_cy[i];
    if (out->cz) out->cz[k] = f->b_cz[i];
    if (out->lambda) out->lambda[k] = f->b_lambda[i];
    if (out->photons) out->photons[k] = f->b_photons[i];
    ++k;
  }
  out->n = k;
  return RBG_OK;
}

}  // extern "C"
