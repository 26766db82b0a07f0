// The saved-state image (.meteolab file) of one run, host side: its header, its layout and its checks, as the
// reference defines them (src/core/state.ts:1-83). Layout: 'MLAB', the JSON header's length (uint32, little endian),
// the JSON header, zero padding to a multiple of 4 bytes, then the fields as float32 in STATE_FIELDS order
// (state.ts:9) and the ground columns in STATE_COLUMNS order (state.ts:10).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

namespace sg {
namespace state {

constexpr int VERSION = 5;        // state.ts:18
constexpr int NSTATE = 22;        // STATE_FIELDS
constexpr int NCOLUMNS = 3;       // STATE_COLUMNS: precipitation, hailGround, hailSize

// Fields a file of this version holds (state.ts:32): 12, 16, 17, 18, 22.
int fields_of(int version);
// The field (sg_field and sg_charge_field ids) behind STATE_FIELDS[k], or -1 for the ones the device step does not
// carry (the two-moment numbers and volumes); the charges (13-16) are an electrified run's.
int carried_of(int k);

struct Info {
  int version = 0, nx = 0, ny = 0, nz = 0, nfields = 0;
  double time = 0, persisted = 0;
  double water[5] = {0, 0, 0, 0, 0};  // the water budget's flows (condensed, evaporated, rainEvaporated, surface) and start
  // chargeGround, flashCount.ic, .cg, charge.separated, .ic, .cgNegative, .cgPositive, .precipitation, .conduction
  double charge[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  size_t data_offset = 0;   // first float of the fields
};

// readState (state.ts:55-68): "" if the image is a state file of a known version whose size matches its grid, else
// the reference's message.
std::string parse(const uint8_t* buf, size_t len, Info& info);

// The version-5 header of saveState (state.ts:43-53) for a run of this grid; `config` is the caller's SimConfig as
// JSON text (null when absent), `water` the budget's condensed, evaporated, rainEvaporated and surface flows and its
// start (the reservoirs' sum when the run began, AtmosphereModel.water.start), `charge` (nullable: zeros) the nine
// numbers of Info::charge.
std::string header_json(const char* config, double time, double persisted, int nx, int ny, int nz, const double water[5],
                        const double* charge = nullptr);

// Whether `text` (null-terminated; null counts as valid) is one JSON value.
bool json_valid(const char* text);

// Bytes of an image with a header of `json_len` bytes, and the offset of its data.
size_t data_offset(size_t json_len);
size_t image_bytes(size_t json_len, int version, int nx, int ny, int nz);

}  // namespace state
}  // namespace sg
