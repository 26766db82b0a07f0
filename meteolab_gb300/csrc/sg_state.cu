// The saved-state image (.meteolab file), host side: the header's JSON, the reference's checks (readState,
// src/core/state.ts:55-68) and the layout. The device side (the fields gathered from and scattered to a run's slot)
// is sg_run_save_state / sg_run_load_state in sg_runtime.cu; sg_state_parse below is the check alone, for hosts
// that want to look at a file before they build the run it belongs to.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include "../../include/stormgpu.h"
#include "sg_state.h"

namespace sg {
namespace state {

namespace {

// A JSON reader that checks the grammar (RFC 8259) and keeps the top-level members the header checks need.
struct Reader {
  const char* p;
  const char* e;
  void ws() { while (p < e && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++; }
  bool lit(const char* s) {
    const size_t n = std::strlen(s);
    if ((size_t)(e - p) < n || std::memcmp(p, s, n) != 0) return false;
    p += n;
    return true;
  }
  bool str(std::string* out) {
    if (p >= e || *p != '"') return false;
    p++;
    while (p < e) {
      const unsigned char c = (unsigned char)*p++;
      if (c == '"') return true;
      if (c < 0x20) return false;
      if (c != '\\') { if (out) out->push_back((char)c); continue; }
      if (p >= e) return false;
      const char d = *p++;
      switch (d) {
        case '"': case '\\': case '/': if (out) out->push_back(d); break;
        case 'b': case 'f': case 'n': case 'r': case 't': if (out) out->push_back(' '); break;
        case 'u':
          for (int k = 0; k < 4; k++, p++) if (p >= e || !std::isxdigit((unsigned char)*p)) return false;
          if (out) out->push_back('?');
          break;
        default: return false;
      }
    }
    return false;
  }
  bool num(double* out) {
    const char* s = p;
    if (p < e && *p == '-') p++;
    if (p >= e || !std::isdigit((unsigned char)*p)) return false;
    if (*p == '0') p++; else while (p < e && std::isdigit((unsigned char)*p)) p++;
    if (p < e && *p == '.') { p++; if (p >= e || !std::isdigit((unsigned char)*p)) return false; while (p < e && std::isdigit((unsigned char)*p)) p++; }
    if (p < e && (*p == 'e' || *p == 'E')) {
      p++;
      if (p < e && (*p == '+' || *p == '-')) p++;
      if (p >= e || !std::isdigit((unsigned char)*p)) return false;
      while (p < e && std::isdigit((unsigned char)*p)) p++;
    }
    if (out) *out = std::strtod(std::string(s, p).c_str(), nullptr);
    return true;
  }
  bool value(int depth) {
    ws();
    if (p >= e || depth > 256) return false;
    switch (*p) {
      case '{': return members(depth, nullptr);
      case '[': {
        p++; ws();
        if (p < e && *p == ']') { p++; return true; }
        for (;;) {
          if (!value(depth + 1)) return false;
          ws();
          if (p < e && *p == ',') { p++; continue; }
          if (p < e && *p == ']') { p++; return true; }
          return false;
        }
      }
      case '"': return str(nullptr);
      case 't': return lit("true");
      case 'f': return lit("false");
      case 'n': return lit("null");
      default: return num(nullptr);
    }
  }
  // An object; `top` (for the header) receives the members it asks for.
  struct Top {
    std::string format;
    bool format_is_string = false;
    double num[6];
    bool is_num[6] = {};
    double water[5] = {0, 0, 0, 0, 0};  // the budget's condensed, evaporated, rainEvaporated, surface, start (absent: 0)
    double charge[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // chargeGround, flashCount ic and cg, the charge budget (absent: 0)
  };
  // A nested object of the header ("water", "flashCount", "charge"): the members named in keys, when numbers, into out.
  bool numbers(int depth, const char* const* keys, int count, double* out) {
    p++; ws();
    if (p < e && *p == '}') { p++; return true; }
    for (;;) {
      ws();
      std::string key;
      if (!str(&key)) return false;
      ws();
      if (p >= e || *p != ':') return false;
      p++; ws();
      bool done = false;
      for (int k = 0; k < count && !done; k++)
        if (key == keys[k] && p < e && (*p == '-' || std::isdigit((unsigned char)*p))) { if (!num(&out[k])) return false; done = true; }
      if (!done && !value(depth + 1)) return false;
      ws();
      if (p < e && *p == ',') { p++; continue; }
      if (p < e && *p == '}') { p++; return true; }
      return false;
    }
  }
  bool members(int depth, Top* top) {
    static const char* keys[6] = {"version", "time", "persisted", "nx", "ny", "nz"};
    p++; ws();
    if (p < e && *p == '}') { p++; return true; }
    for (;;) {
      ws();
      std::string key;
      if (!str(&key)) return false;
      ws();
      if (p >= e || *p != ':') return false;
      p++; ws();
      bool done = false;
      if (top) {
        static const char* waterKeys[5] = {"condensed", "evaporated", "rainEvaporated", "surface", "start"};
        static const char* flashKeys[2] = {"ic", "cg"};
        static const char* chargeKeys[6] = {"separated", "ic", "cgNegative", "cgPositive", "precipitation", "conduction"};
        if (key == "water" && p < e && *p == '{') { if (!numbers(depth + 1, waterKeys, 5, top->water)) return false; done = true; }
        if (key == "flashCount" && p < e && *p == '{') { if (!numbers(depth + 1, flashKeys, 2, top->charge + 1)) return false; done = true; }
        if (key == "charge" && p < e && *p == '{') { if (!numbers(depth + 1, chargeKeys, 6, top->charge + 3)) return false; done = true; }
        if (key == "chargeGround" && p < e && (*p == '-' || std::isdigit((unsigned char)*p))) { if (!num(&top->charge[0])) return false; done = true; }
        if (key == "format") {
          if (p < e && *p == '"') { std::string v; if (!str(&v)) return false; top->format = v; top->format_is_string = true; done = true; }
          else top->format_is_string = false;
        }
        for (int k = 0; k < 6 && !done; k++) {
          if (key != keys[k]) continue;
          if (p < e && (*p == '-' || std::isdigit((unsigned char)*p))) { if (!num(&top->num[k])) return false; top->is_num[k] = true; done = true; }
          else top->is_num[k] = false;  // a later duplicate key wins, as in JSON.parse
        }
      }
      if (!done && !value(depth + 1)) return false;
      ws();
      if (p < e && *p == ',') { p++; continue; }
      if (p < e && *p == '}') { p++; return true; }
      return false;
    }
  }
};

// A number as JavaScript's JSON.stringify writes integers, other values with 17 significant digits.
std::string js_number(double v) {
  char b[40];
  if (!std::isfinite(v)) return "null";
  if (v == std::floor(v) && std::fabs(v) < 1e15) std::snprintf(b, sizeof b, "%.0f", v);
  else std::snprintf(b, sizeof b, "%.17g", v);
  return b;
}

}  // namespace

int fields_of(int version) { return version == 1 ? 12 : version == 2 ? 16 : version == 3 ? 17 : version == 4 ? 18 : 22; }

int carried_of(int k) {
  // STATE_FIELDS (state.ts:9): u v w theta q cloud rain cold ice snow graupel hail, chargeIce chargeGraupel chargeRain
  // chargeAir, iceNumber, rainNumber, graupelNumber graupelVolume hailNumber hailVolume
  static const int map[NSTATE] = {SG_U, SG_V, SG_W, SG_THETA, SG_Q, SG_CLOUD, SG_RAIN, SG_COLD, SG_ICE, SG_SNOW, SG_GRAUPEL, SG_HAIL,
                                  SG_CHARGE_ICE, SG_CHARGE_GRAUPEL, SG_CHARGE_RAIN, SG_CHARGE_AIR, SG_ICE_NUMBER, SG_RAIN_NUMBER,
                                  SG_GRAUPEL_NUMBER, SG_GRAUPEL_VOLUME, SG_HAIL_NUMBER, SG_HAIL_VOLUME};
  return k >= 0 && k < NSTATE ? map[k] : -1;
}

size_t data_offset(size_t json_len) { return (8 + json_len + 3) / 4 * 4; }

size_t image_bytes(size_t json_len, int version, int nx, int ny, int nz) {
  const size_t cells = (size_t)nx * ny;
  return data_offset(json_len) + ((size_t)fields_of(version) * cells * nz + (size_t)NCOLUMNS * cells) * 4;
}

std::string parse(const uint8_t* buf, size_t len, Info& info) {
  if (!buf || len < 8 || std::memcmp(buf, "MLAB", 4) != 0) return "this is not a MeteoLab state file";
  const uint32_t length = (uint32_t)buf[4] | (uint32_t)buf[5] << 8 | (uint32_t)buf[6] << 16 | (uint32_t)buf[7] << 24;
  if (8 + (uint64_t)length > len) return "the file is truncated";
  Reader r{reinterpret_cast<const char*>(buf) + 8, reinterpret_cast<const char*>(buf) + 8 + length};
  Reader::Top top;
  r.ws();
  bool ok;
  if (r.p < r.e && *r.p == '{') ok = r.members(0, &top);
  else ok = r.value(0);  // any other JSON value: valid, but not a header
  r.ws();
  if (!ok || r.p != r.e) return "the file's header is damaged";
  const double version = top.num[0];
  if (top.format != "meteolab-state" || !top.format_is_string || !top.is_num[0] ||
      !(version == 1 || version == 2 || version == 3 || version == 4 || version == 5))
    return "unknown file format or version";
  for (int k = 1; k < 6; k++)
    if (!top.is_num[k] || !std::isfinite(top.num[k]) || top.num[k] < 0) return "the file's header is damaged";
  for (int k = 3; k < 6; k++)  // a grid of whole, addressable sizes
    if (top.num[k] != std::floor(top.num[k]) || top.num[k] > 1e6) return "the file's header is damaged";
  info.version = (int)version;
  info.time = top.num[1]; info.persisted = top.num[2];
  info.nx = (int)top.num[3]; info.ny = (int)top.num[4]; info.nz = (int)top.num[5];
  info.nfields = fields_of(info.version);
  for (int k = 0; k < 5; k++) info.water[k] = top.water[k];
  for (int k = 0; k < 9; k++) info.charge[k] = top.charge[k];
  info.data_offset = data_offset(length);
  if (len != image_bytes(length, info.version, info.nx, info.ny, info.nz)) return "the file's size does not match the grid";
  return "";
}

std::string header_json(const char* config, double time, double persisted, int nx, int ny, int nz, const double water[5], const double* charge) {
  static const double none[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const double* c = charge ? charge : none;
  std::string j = "{\"format\":\"meteolab-state\",\"version\":" + std::to_string(VERSION) + ",\"config\":";
  j += config && *config ? config : "null";
  j += ",\"time\":" + js_number(time) + ",\"persisted\":" + js_number(persisted);
  j += ",\"nx\":" + std::to_string(nx) + ",\"ny\":" + std::to_string(ny) + ",\"nz\":" + std::to_string(nz);
  j += ",\"chargeGround\":" + js_number(c[0]) + ",\"flashCount\":{\"ic\":" + js_number(c[1]) + ",\"cg\":" + js_number(c[2]) + "}";
  j += ",\"water\":{\"condensed\":" + js_number(water[0]) + ",\"evaporated\":" + js_number(water[1]) + ",\"rainEvaporated\":" +
       js_number(water[2]) + ",\"surface\":" + js_number(water[3]) + ",\"start\":" + js_number(water[4]) + "}";
  j += ",\"added\":{\"heat\":0,\"vapour\":0,\"count\":0}";
  j += ",\"charge\":{\"separated\":" + js_number(c[3]) + ",\"ic\":" + js_number(c[4]) + ",\"cgNegative\":" + js_number(c[5]) +
       ",\"cgPositive\":" + js_number(c[6]) + ",\"precipitation\":" + js_number(c[7]) + ",\"conduction\":" + js_number(c[8]) + "}}";
  return j;
}

bool json_valid(const char* text) {
  if (!text) return true;
  Reader r{text, text + std::strlen(text)};
  const bool ok = r.value(0);
  r.ws();
  return ok && r.p == r.e;
}

}  // namespace state
}  // namespace sg

extern "C" int sg_state_parse(const uint8_t* image, size_t len, sg_state_info* out, char* err, size_t err_len) {
  sg::state::Info info;
  const std::string msg = sg::state::parse(image, len, info);
  if (!msg.empty()) {
    if (err && err_len) std::snprintf(err, err_len, "%s", msg.c_str());
    return SG_ERR_INVALID;
  }
  if (out) {
    out->version = info.version; out->nx = info.nx; out->ny = info.ny; out->nz = info.nz; out->nfields = info.nfields;
    out->time = info.time; out->persisted = info.persisted; out->data_offset = (uint64_t)info.data_offset;
  }
  if (err && err_len) err[0] = 0;
  return SG_OK;
}
