// Launch parameters of the adjoint kernels (plain structs, no device code).
#pragma once
#include "sf_forward.cuh"

namespace sf {

struct AdjParams {
    int nzz, nxx, nb;
    float dx, dz;
    const ShotDev* shots;   // same table (and order) as the taped forward
    int nshots;
    int nstrips;
    int G, NG, maxcols;     // gangs as in the forward
    float* lam;             // per-gang window adjoint, lam + gang * lam_per_gang
    long long lam_per_gang;
    unsigned long long* hand;  // per gang [4][nstrips][2 * maxcols] tagged (pv, pev) pairs
    unsigned* bar;          // per gang barrier counter
    unsigned epoch;         // launch number (tags)
    unsigned long long wait_ns;  // time limit of the bounded waits
    uint8_t* tcode;
    float* tc1;
    float* tc2;
    const float* pick_grad; // nshots x nrec, caller order (NaN = no pick)
    const float* rx;
    const float* rz;
    int nrec;
    float* lam_init;        // nshots x 9, caller order: adjoint of the 3x3 initial values
    int* err;
    // seed table: node n (row seed_row[n], padded column seed_col[n]) gets, in
    // receiver order, pick_grad[r] * seed_w[e] for entries e of
    // [seed_ptr[n], seed_ptr[n+1]) whose receiver r = seed_rec[e] has its
    // stencil inside the shot's window (column rec_jg[r] - c0)
    int nseed;
    const int* seed_ptr;
    const int* seed_row;
    const int* seed_col;
    const int* seed_rec;
    const int* rec_jg;
    const float* seed_w;
};

// A shot as the gather sees it: one entry per (column block, shot covering
// it), caller order within a block.
struct GatherShot {
    long long tape_off;
    int c0, ncols;
    int sIdx, sIdz;
    float sx, sz;
    int orig, pad_;
    long long q_off;        // the shot's qP derivative factors (anisotropic batches)
};

struct GatherParams {
    int nzz, nxx, nb, nstrips, nshots;
    const int* blk_ptr;            // entries of column block cb: [blk_ptr[cb], blk_ptr[cb+1])
    const GatherShot* blk_shots;
    float dx, dz;
    const uint8_t* tcode;
    const float* vrec;       // v terms (tape c2 after the reverse sweeps)
    const float* lam_init;   // nshots x 9 (caller order)
    float* grad;             // nzz x nxx
    // anisotropic batches: each shot's gradient with respect to its qP
    // slowness, times the shot's dSq/dS, dSq/dC11, dSq/dC13 (3 x vfac_total)
    const float* vfac;
    long long vfac_total;
    float* grad_c11;         // nzz x nxx
    float* grad_c13;         // nzz x nxx
    // gather inside the reverse-sweep launch: a shot's initialisation term is
    // final when shot_done[orig] == done_tag; waits give up with *err set
    const unsigned* shot_done;
    unsigned done_tag;
    int* err;
    unsigned long long wait_ns;  // time limit of the bounded waits
};

// The reverse sweeps and the gather in one launch: CTAs [0, nadj) run the
// reverse sweeps and count, per (strip, column block), the shots whose last
// reverse sweep has finished the block (ready); the other CTAs take tiles in
// that order (tile_ctr) and start a tile when every shot covering it has
// finished it in the tile's strip and the next one.
struct FuseParams {
    int nadj;            // reverse-sweep CTAs
    int nblk;            // column blocks of kGT columns
    unsigned* ready;     // nstrips x nblk counters (zeroed per launch)
    unsigned* tile_ctr;  // next tile (zeroed per launch)
    unsigned* shot_done; // per shot: done_tag once its initialisation term is written
    unsigned done_tag;
};

}  // namespace sf
