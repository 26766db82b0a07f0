// The copy plan of the bulk-copy transport tiles (sg_transport.cu): which cp.async.bulk row copies fill a tile's
// shared-memory packet of one level, as plain index arithmetic usable on the host too (the CPU tests enumerate every
// copy of the benchmark grids and check bounds, 16-byte alignment, coverage and the announced byte count).
//
// A packet of level L holds (a) planes of the G fields (the ring: PH = TY + 6 rows of PW = TX + 8 floats, the periodic
// window [x0 - 4, x0 + TX + 4) x [y0 - 3, y0 + TY + 3) of one level), and (b) the level's auxiliary rows: the tile's
// face fluxes (float4 per column, TY rows of TX), the west edge's faces (one float4 per tile row), the south edge's
// faces (a row of TX float4), and for the WENO fields the step-start values of the G fields (TY rows of TX floats).
#pragma once
#include "sg_common.cuh"

namespace sg {

struct TileCopies {
  int nx, ny, layer, TX, TY, x0, y0, G;
  bool s0;  // the step-start values travel in the packet
  SG_HD int PW() const { return TX + 8; }
  SG_HD int PH() const { return TY + 6; }
  SG_HD int rows_on() const { return TY < ny - y0 ? TY : ny - y0; }
  SG_HD int ncols() const { return TX < nx - x0 ? TX : nx - x0; }
  // piece k of a window row: smem column c, global column gx, length l (floats)
  SG_HD void piece(int k, int& c, int& gx, int& l) const {
    c = 0;
    for (int q = 0;; q++) {
      gx = wrap(x0 - 4 + c, nx);
      l = PW() - c < nx - gx ? PW() - c : nx - gx;
      if (q == k) return;
      c += l;
    }
  }
  // the number of pieces of a row (at most three) and the columns they cover (PW when TX <= nx)
  SG_HD int pieces(int& covered) const {
    int k = 0;
    covered = 0;
    while (covered < PW() && k < 3) { int c, gx, l; piece(k, c, gx, l); covered = c + l; k++; }
    return k;
  }
  // ring copy j < PH * nseg of one plane: smem float offset in the plane, global float offset from the plane's level
  // start, length in floats
  SG_HD void ring(int j, int nseg, int& soff, int& goff, int& len) const {
    const int r = j / nseg, k = j - r * nseg;
    const int gy = ((y0 - 3 + r) % ny + ny) % ny;
    int c, gx;
    piece(k, c, gx, len);
    soff = r * PW() + c;
    goff = gy * nx + gx;
  }
  // auxiliary copies of a level
  SG_HD int naux() const { return 2 * rows_on() + 1 + (s0 ? G * rows_on() : 0); }
  SG_HD int aux_floats() const { return 4 * (TY * TX + TY + TX) + (s0 ? G * TY * TX : 0); }
  // auxiliary copy j: smem float offset in the packet's auxiliary buffer; the source as a float4 index from the level
  // start of the face fluxes (which = 0) or a float index from the level start of step-start field g (which = 1 + g);
  // length in bytes
  SG_HD void aux(int j, int& soff, int& src, int& which, int& bytes) const {
    const int ro = rows_on(), nc = ncols();
    if (j < ro) { soff = 4 * j * TX; src = x0 + (y0 + j) * nx; which = 0; bytes = 16 * nc; }
    else if (j < 2 * ro) { const int r = j - ro; soff = 4 * (TY * TX + r); src = wrap(x0 - 1, nx) + (y0 + r) * nx; which = 0; bytes = 16; }
    else if (j == 2 * ro) { soff = 4 * (TY * TX + TY); src = x0 + wrap(y0 - 1, ny) * nx; which = 0; bytes = 16 * nc; }
    else {
      const int k = j - 2 * ro - 1, g = k / ro, r = k - g * ro;
      soff = 4 * (TY * TX + TY + TX) + (g * TY + r) * TX; src = (y0 + r) * nx + x0; which = 1 + g; bytes = 4 * nc;
    }
  }
  // bytes of a packet with `planes` ring planes
  SG_HD unsigned bytes(int planes) const {
    int covered;
    pieces(covered);
    const int ro = rows_on(), nc = ncols();
    return (unsigned)(planes * G * PH() * covered * 4) + (unsigned)(ro * 16 * nc + ro * 16 + 16 * nc) + (s0 ? (unsigned)(G * ro * 4 * nc) : 0u);
  }
};

}  // namespace sg
