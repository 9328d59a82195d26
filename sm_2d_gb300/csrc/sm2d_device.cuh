// sm2d_device.cuh -- device-side physics, slot tables and bin encodings of
// the transport step.  Float arithmetic follows the reference's expression
// order (device_physics.cuh, device_lut.cuh, device_bucket.cuh,
// device_psic.cuh); exp/log/sin/cos/erf come from sm2d_math.h, which the CPU
// oracle shares, so per-bin results are bit-identical to the oracle's and
// within about an ulp of the reference build's.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "sm2d.h"
#include "sm2d_math.h"

namespace sm2d {

constexpr uint32_t kEmpty = 0xFFFFFFFFu;
constexpr int kKb = 32;
constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr int kMaxLanes = 512;   // per-lane sums are staged in shared memory

// One beam on the device (sm2d_beam).  kind 0: the runner's source (pencil
// or LCG Gaussian, n samples); kind 1: the quadrature source, n samples over
// the q_nx cells from q_ix0 (the host computes the cell range).
struct BeamArgs {
    float x0, z0, theta0, E0, W, sx, sth, sE;
    int n;
    unsigned seed;
    int kind, q_ix0, q_nx;
};

// Local-bin layout: lidx = t + NT*(e + NE*(x + NX*z))  (local_bins.hpp:62-78)
template <int NT_, int NE_, int NX_, int NZ_>
struct Layout {
    static constexpr int NT = NT_, NE = NE_, NX = NX_, NZ = NZ_;
    static constexpr int L = NT * NE * NX * NZ;
    __device__ __forceinline__ static int enc(int t, int e, int x, int z) { return t + NT * (e + NE * (x + NX * z)); }
    __device__ __forceinline__ static void dec(int l, int& t, int& e, int& x, int& z) {
        t = l % NT;
        int r = l / NT;
        e = r % NE;
        r /= NE;
        x = r % NX;
        z = r / NX;
    }
};
using LayoutRef = Layout<4, 2, 8, 4>;    // 256 bins: the layout the reference code builds
using LayoutB128 = Layout<8, 4, 4, 1>;   // 128 bins: 8 theta x 4 E x 4 x_sub

// The engine holds B lanes: B independent spots, each with its own grid of
// Nc cells, stacked so that every per-cell array is indexed by
// gc = lane * Nc + cell.  All lanes advance together, one transport
// iteration per pass of the kernel sequence; a lane without work idles.

// Iteration state shared by the lanes (one per engine), written only by
// device code between host syncs.
// Drop counters of k2/k3/k4_get_debug_counters (k2_coarsetransport.cuh:101-112,
// k3_finetransport.cuh:78-89, k4_transfer.cuh:19-24): per stage (K2, K3, K4)
// and kind (output slot, bucket, prune), the dropped components, their
// weight and energy, since the last reset.
enum { DROP_SLOT = 0, DROP_BUCKET = 1, DROP_PRUNE = 2 };
struct DropCounters {
    unsigned long long n[3][3];
    double w[3][3], e[3][3];
};

struct IterGlobal {
    int parity;            // occupancy list `parity` lists psi_in, `parity ^ 1` psi_out
    int halt;              // this pass does no transport (no lane has work, or paused)
    int pass;              // transport passes done since the last reset
    int max_pass;          // the device loop pauses after this many passes
    unsigned blocks_done;  // last-block counter of the classify and finalize kernels
    int occ_n[2];          // length of each occupancy list
    int n_listed;          // cells of this pass (active + coarse, all lanes)
    int n_items;           // claimed slots of the listed cells
    int n_bins;            // w > 0 local bins of the listed cells (transport work)
    unsigned long long acc_lb;   // classify: listed cells << 32 | their w > 0 bins (one reservation a cell)
    int pool_peak;         // the most value pages one lane held (since the last reset)
    int bin_ovf;           // the cell list, bin list or a lane's value pages outgrew their capacity
                           // (since the last reset)
    int cand_ovf;          // claim-table inserts that found no free entry (cumulative)
    int cand_miss;         // deposits whose block id was not gathered (cumulative)
    int wipe;              // claim tables are cleared before the next pass
    int k3_rows;           // surrogate rows asked for by this pass's claim pass (may pass k3_cap)
    int k3_ovf;            // K3 bins past the rows' capacity (closed forms; cumulative)
    unsigned long long k3_total;   // surrogate rows served by earlier passes since the last reset
    unsigned long long k3_fb;      // of those, rows that fell back to the closed forms
    uint32_t ctag;         // claim pass number: the tag of claim-table entries
    unsigned long long gen;  // K1 classifications done since create (never reset)
    // spot plan (sm2d_batch_run): lanes that finish take the plan's next
    // spot inside the device loop; plan_n == 0 outside a plan
    int plan_n;            // spots of the plan
    int lane_limit;        // lanes 0 .. lane_limit - 1 take the plan's spots (0: every lane)
    int plan_next;         // next spot to hand out
    int lane_max_it;       // iteration limit of one spot
    int refills;           // refill rounds run
    unsigned long long bins_total;   // bins transported since the last reset
    int occ_mark;          // psi_in's occupancy list length when the injection opened
    int n_fin;             // lanes whose spot finished at this classification
    int fin[kMaxLanes];    // those lanes, ascending
    int n_fill;            // lanes the last refill assigned, and their spots
    int fill_lane[kMaxLanes], fill_spot[kMaxLanes];
    const BeamArgs* plan_beams;   // [plan_n]
    const int* plan_order;        // [plan_n]: the spots in the order lanes take them (longest first)
    const float* plan_fe;         // [plan_n][3 Nz + 1]: A(z), B(z), sigma_total(z), sigma_x
    double* plan_dose;            // [plan_n][Nc] convolved dose, or null
    sm2d_spot_result* plan_res;   // [plan_n]
    DropCounters drops;           // cleared with the iteration state
};

// One dropped component (rare paths only): stage 0 K2, 1 K3, 2 K4.  Out of
// line, so that the emission code inlined at many sites stays small.
static __device__ __noinline__ void count_drop(IterGlobal* gs, int stage, int kind, double w, double e) {
    atomicAdd(&gs->drops.n[stage][kind], 1ull);
    atomicAdd(&gs->drops.w[stage][kind], w);
    atomicAdd(&gs->drops.e[stage][kind], e);
}

// Per-lane (per-spot) state.
struct LaneState {
    int iter;              // transport iterations of this lane's spot
    int n_active, n_coarse;
    int done;              // no listed cell: transport finished (or nothing injected)
    int include_source;    // next audit lifts source losses (first iteration)
    int work;              // this pass transports this lane
    int light;             // stopping rule met at the start of this pass
    int acc_active, acc_coarse, acc_slots;   // classify counters
    int inj_skip;          // the last injection found the lane occupied
    int w_fail, e_fail;    // iterations whose weight / energy audit failed
    int spot;              // plan spot in this lane (-1: none)
    int refill;            // the next injection fills this lane
    int stopped;           // the spot reached the iteration limit of a plan
    // value pages of this lane's region handed out since its psi_in was
    // last consumed
    int pool_top, pad2;
    // per-iteration accumulators, 14 consecutive doubles (reset by the
    // classify kernel); the transport adds to the first seven, the finalize
    // kernel to the last seven, in this order
    double drop_w, drop_e, Win, Ein, Wout, Eout, slots_out_it;
    double Edep, Ecut, Enuc, Ebnd, Wcut, Wnuc, Wbnd;
    // cumulative
    double transport_drop_w, transport_drop_e, audit_residual;
    double cell_steps, slots_in, slots_out;
    // source accounting
    float src_inj_w, src_oog_w, src_slot_w, pad1;
    double src_inj_e, src_oog_e, src_slot_e, src_rep_loss;
    double tot_w, tot_e;   // scratch for phase-space totals
    sm2d_audit last;
};

struct Dev {
    int Nx, Nz, Nc;       // grid of one lane
    int B;                // lanes
    float dx, dz;
    int N_theta, N_E;
    const float* th;      // theta edges [N_theta+1]
    const float* Ee;      // energy edges [N_E+1]
    int lutN;
    float lutEmin, lutEmax;
    const float *R, *logE, *logR;
    float R_fine_on;      // lut_range(max(E_fine_on, lutEmin)), evaluated once on the device
    // per energy bin, K2 at the bin-centre energy over the coarse step in a
    // row of density 1 whose step does not split at the fine threshold:
    // range, energy loss, nuclear survival, scattering power (the transport's
    // own arithmetic, evaluated once on the device) [N_E]
    const float4* k2tab;
    // search tables (slot_of): the energy bin / R index where the searches
    // of the slot's smallest value end
    const int *e_slot, *r_slot;
    uint32_t e_base, r_base;
    int e_nslot, r_nslot;
    // per lane: Fermi-Eyges moments A(z), B(z), sigma_total(z) [B][Nz] of the
    // lane's beam (k1k6_pipeline.cu:1061-1206) and its initial sigma_x [B]
    float *feA, *feB, *feS, *sx0;
    // slab phantom: density of each depth row and the water-equivalent depth
    // of each row's upper face [Nz]; null for water
    const float *rho, *wet;
    float E_fine_on, wmin, step_coarse;
    int b_on, b_off;
    int straggle, nuclear, seed_mode, esplit;
    float prune_coarse, prune_fine, split_min_w, stop_frac;
    int floor_cutoff, salt;
    // phase space: ids [B * Nc][32]; values in pages of L floats.  A cell's
    // claimed slots hold consecutive pages from pbase[gc] on (slot s in page
    // pbase[gc] + s); the psi_out selection hands each cell its run from the
    // lane's region [lane * pool_lane, (lane + 1) * pool_lane), and pages
    // pool_lane * B .. + 31 take the writes of a cell whose lane ran out
    // (the run stops with SM2D_ERR_ALLOC).  The classify kernel copies
    // psi_in into the bin list and clears its pages, so free pages hold
    // zeros and the lane's region is handed out again from its start.
    uint32_t* bid;
    float* val;
    int* pbase;           // [B * Nc]: first page of the cell's slots
    int pool_lane;        // pages per lane
    // per page, one bit per float4 of its values (L / 4 <= 64 bits, two
    // words): set by every writer of a value, so a clear bit means four zero
    // values; the classify kernel reads only the marked float4s and clears
    // the bits with them
    uint2* vmask;
    int* occ[2];          // per gc: on occupancy list k
    int* occ_list[2];     // occupancy lists (gc), in claim order
    int* occ_pg[2];       // first value page of each listed cell (its pbase), set with the pages
    double *edep, *e_cut, *e_nuc, *e_bnd;
    float *w_cut, *w_nuc, *w_bnd;
    // this iteration's per-cell tally increments (folded into the cumulative
    // tallies with the audit's per-cell clamp by the finalize kernel)
    double *dl_edep, *dl_ecut, *dl_enuc, *dl_ebnd;
    float *dl_wcut, *dl_wnuc, *dl_wbnd;
    // K1 mask as the number of the last classification that found the cell
    // active: bit 0 of the reference mask is act_gen == gen, its hysteresis
    // input ("was active") is act_gen == gen - 1 at the next classification
    unsigned long long* act_gen;
    uint8_t* cls;         // 0 idle, 1 coarse (K2), 2 active (K3); 0 outside the iteration
    uint32_t* listed;     // this pass's active + coarse cells (gc, claim order)
    int listed_cap;
    uint4* bins;          // w > 0 bins of the listed cells, grouped by cell:
                          // {gc, slot | seed slot << 5 | lidx << 10 | K3 << 18, w bits, block id}
    uint4* brec;          // per bin, two uint4: the step's outcome from the claim pass
    float4* brec2;        // expectation form, per bin: sigma_theta / dtheta, straggling sigma,
                          // the bin's row of the surrogate's tables (int bits, -1: none)
    int expect;           // 1: expectation form (redistribution weights instead of draws)
    // precision form: weight tallies booked as increments in the audit, the
    // R-LUT inverted in double below R_prec = lut_range(10 MeV)
    int precise;
    float R_prec;
    // expectation form with the learned surrogate: the claim pass gives each
    // K3 bin inside the network's domain a row (its feature row (s, u, r,
    // cap) and its bin-list entry) and leaves its claims for later; the
    // network fills the rows' tables [32] and fallback flags; the rows' claim
    // pass and the deposit pass then emit from the table, or from the closed
    // forms where the row fell back [k3_cap]
    int surr, k3_cap;
    float4* kfeat;
    int* kbin;
    float* ktab;
    int* kfb;
    int2* cell_bins;      // per listed cell: its first bin and bin count in the bin list
    int bins_cap;
    uint32_t *active, *coarse;   // ascending lists of lane 0 (built on request by k_order_lists)
    IterGlobal* gs;
    LaneState* ls;        // [B]
    sm2d_audit* hist;     // [B][hist_cap]
    int hist_cap;
    unsigned char* buckets;  // DeviceOutflowBucket array (bucket mode) [4 * listed_cap]
    int* c2b;                // listed gc -> bucket base 4 * list position, -1 otherwise
    int bucket_bytes;
    unsigned long long* ctab;  // claim tables: B * Nc psi_out rows, then 4 * listed_cap bucket rows
    int* ccount;               // gathered ids per claim-table row
    uint32_t* bkt_ids;         // kept ids of each bucket row [4 * listed_cap][32]
    // per kept bucket id (bucket row, position): the value page of its psi_out
    // slot in the cell behind the face and that slot's id (bkt_slot_pack),
    // resolved once per pass by the selection [4 * listed_cap][32]
    uint2* bkt_os;
};

__device__ __forceinline__ int lane_of(const Dev& d, int gc) { return gc / d.Nc; }

// ---------------------------------------------------------------- encodings
__device__ __forceinline__ uint32_t make_bid(uint32_t bt, uint32_t be) { return (bt & 0xFFFu) | ((be & 0xFFFu) << 12); }
__device__ __forceinline__ float sub_offset(int s, int n, float d) { return d * ((0.5f + (float)s) / (float)n - 0.5f); }
__device__ __forceinline__ int sub_bin(float off, float d, int n) {
    int b = (int)(((off / d) + 0.5f) * (float)n);
    return b < 0 ? 0 : (b >= n ? n - 1 : b);
}

// ---------------------------------------------------------------- LUT (device_lut.cuh:34-214)
// The searches of the LUT (device_find_bin_edges, the R inversion) start
// from a table indexed by the top bits of the value's float pattern
// (2^(23 - kSlotShift) slots per octave, monotone in the value): the
// table holds the search result at the slot's smallest value, a lower bound
// for every value in the slot, and a forward scan of a few entries ends at
// exactly the binary search's result.
constexpr int kSlotShift = 15;
__device__ __forceinline__ int slot_of(float x, uint32_t base, int n) {
    const int j = (int)(__float_as_uint(x) >> kSlotShift) - (int)base;
    return max(0, min(j, n - 1));
}
// bin b of the energy edges with Ee[b] <= E < Ee[b+1], clamped to [0, N_E)
__device__ __forceinline__ int find_ebin(const Dev& d, float E) {
    const float* e = d.Ee;
    if (E <= e[0]) return 0;
    if (E >= e[d.N_E]) return d.N_E - 1;
    int b = d.e_slot[slot_of(E, d.e_base, d.e_nslot)];
    while (e[b + 1] <= E) ++b;   // stops at N_E - 1 at the latest: E < e[N_E]
    return b;
}
__device__ __forceinline__ float lut_range(const Dev& d, float E) {
    float Ec = fmaxf(d.lutEmin, fminf(E, d.lutEmax));
    int b = find_ebin(d, Ec);
    if (b == d.lutN - 1 || Ec >= d.lutEmax) return d.R[d.lutN - 1];
    float le = sm2d_logf(Ec);
    float lr = d.logR[b] + (d.logR[b + 1] - d.logR[b]) * (le - d.logE[b]) / (d.logE[b + 1] - d.logE[b]);
    return sm2d_expf(lr);
}
__device__ __forceinline__ float lut_energy_of_range(const Dev& d, float r) {
    if (r <= 0.0f) return d.lutEmin;
    int lo = d.r_slot[slot_of(r, d.r_base, d.r_nslot)];   // first index with R[lo] >= r
    while (lo < d.lutN && d.R[lo] < r) ++lo;
    int b = max(0, min(lo, d.lutN - 2));
    if (d.precise && r < d.R_prec) {   // precision form: the interpolation in double below 10 MeV
        const double dl = (double)d.logR[b + 1] - (double)d.logR[b];
        if (fabs(dl) < 1e-10) return (float)exp((double)d.logE[b]);
        const double le =
            (double)d.logE[b] + ((double)d.logE[b + 1] - (double)d.logE[b]) * (log((double)r) - (double)d.logR[b]) / dl;
        return (float)exp(le);
    }
    float lr = sm2d_logf(r);
    float dl = d.logR[b + 1] - d.logR[b];
    if (fabsf(dl) < 1e-10f) return sm2d_expf(d.logE[b]);
    float le = d.logE[b] + (d.logE[b + 1] - d.logE[b]) * (lr - d.logR[b]) / dl;
    return sm2d_expf(le);
}
// energy lost over path s from E, whose range RE = lut_range(d, E)
__device__ __forceinline__ float lut_energy_loss(const Dev& d, float E, float RE, float s) {
    float r = RE - s;
    float En = (r <= 0.0f) ? d.lutEmin : lut_energy_of_range(d, r);
    return E - En;
}
// K3 step limit at E, whose range RE = lut_range(d, E)
__device__ __forceinline__ float fine_step_limit(float E, float RE) {
    float v = 0.01f * RE;
    float floor_ = E < 2.0f ? 0.1f : (E < 20.0f ? 0.25f : (E < 100.0f ? 0.5f : 1.0f));
    v = fmaxf(v, floor_);
    if (E < 0.5f) v = fminf(v, 0.05f);
    else if (E < 5.0f) v = fminf(v, 0.2f);
    else if (E < 20.0f) v = fminf(v, 0.5f);
    return v;
}

// ---------------------------------------------------------------- physics (device_physics.cuh)
constexpr float kMp = 938.272f, kMe = 0.511f, kX0 = 360.8f;

__device__ __forceinline__ float highland(float E, float ds) {
    float g = (E + kMp) / kMp;
    float b2 = 1.0f - 1.0f / (g * g);
    float beta = sqrtf(fmaxf(b2, 0.0f));
    float p = sqrtf(fmaxf((E + kMp) * (E + kMp) - kMp * kMp, 0.0f));
    float t = ds / kX0;
    if (t < 1e-6f) return 0.0f;
    float br = fmaxf(1.0f + 0.038f * sm2d_logf(t), 0.25f);
    return (13.6f * 1.0f / (beta * p)) * sqrtf(t) * br;
}
// scattering power per geometric mm in a medium of density rho: the
// Highland angle of the water-equivalent thickness rho ds
__device__ __forceinline__ float scatter_power(float E, float ds, float rho) {
    float th = highland(E, rho * ds);
    if (ds < 1e-6f) return 0.0f;
    return th * th / ds;
}
// LCG + Box-Muller draw of the transport kernels
__device__ __forceinline__ float normal_draw(unsigned& s) {
    s = 1664525u * s + 1013904223u;
    float u1 = (float)(s >> 16) / 65536.0f;
    s = 1664525u * s + 1013904223u;
    float u2 = (float)(s >> 16) / 65536.0f;
    u1 = fmaxf(u1, 1e-6f);
    return sqrtf(-2.0f * sm2d_logf(u1)) * sm2d_cosf(2.0f * 3.14159265358979323846f * u2);
}
__device__ __forceinline__ float vav_xi(float beta, float rho, float ds_cm) {
    return (0.307f / 2.0f) * 0.555f * (1.0f * 1.0f / (beta * beta)) * rho * ds_cm;
}
__device__ __forceinline__ float bohr_sigma(float E, float ds, float rho) {
    float g = (E + kMp) / kMp;
    float beta = sqrtf(fmaxf(1.0f - 1.0f / (g * g), 0.01f));
    return 0.156f * sqrtf(rho * ds) / beta;
}
__device__ __forceinline__ float straggling_sigma(float E, float ds, float rho) {
    float g = (E + kMp) / kMp;
    float beta = sqrtf(fmaxf(1.0f - 1.0f / (g * g), 0.0f));
    float xi = vav_xi(beta, rho, ds / 10.0f);
    float mr = kMe / kMp;
    float tmax = (2.0f * kMe * beta * beta * g * g) / fmaxf(1.0f + 2.0f * g * mr + mr * mr, 1e-10f);
    float kappa = fmaxf(xi / fmaxf(tmax, 1e-10f), 1e-6f);
    if (kappa > 10.0f) return bohr_sigma(E, ds, rho);
    float landau = 4.0f * xi / 2.355f;
    if (kappa < 0.01f) return landau;
    float w = 1.0f / (1.0f + kappa);
    return w * landau + (1.0f - w) * bohr_sigma(E, ds, rho);
}
__device__ __forceinline__ float nuclear_xs(float E) {
    if (E < 5.0f) return 0.0f;
    if (E >= 20.0f) return 0.0012f * fmaxf(1.0f - 0.15f * sm2d_logf(E / 100.0f), 0.4f);
    return 0.0016f * ((E - 5.0f) / 15.0f);
}
__device__ __forceinline__ float gauss_cdf(float x, float mu, float sigma) {
    if (sigma < 1e-10f) return (x >= mu) ? 1.0f : 0.0f;
    const float dd = x - mu;
    // beyond 8 sigma the argument of erf exceeds 4, where sm2d_erff is
    // exactly +-1: the same 1 or 0 without the division and the series
    if (dd > 8.0f * sigma) return 1.0f;
    if (dd < -8.0f * sigma) return 0.0f;
    float c = 0.5f * (1.0f + sm2d_erff(dd / sigma * 0.70710678f));
    return fminf(1.0f, fmaxf(0.0f, c));
}

// ---------------------------------------------------------------- slot tables
__device__ __forceinline__ int bid_distance(uint32_t a, uint32_t b) {
    int ta = (int)(a & 0xFFFu), ea = (int)((a >> 12) & 0xFFFu);
    int tb = (int)(b & 0xFFFu), eb = (int)((b >> 12) & 0xFFFu);
    return abs(ea - eb) * 8 + abs(ta - tb);
}
// exact match, then CAS-claim an empty slot, then nearest occupied block
// (device_psic.cuh:208-260 and device_bucket.cuh:61-128, same protocol);
// used by the K4 stage entry on caller arrays.
__device__ __forceinline__ int claim_slot(uint32_t* ids, uint32_t want, uint32_t& sel) {
    sel = want;
    volatile uint32_t* v = ids;
    for (int s = 0; s < kKb; ++s)
        if (v[s] == want) return s;
    for (int s = 0; s < kKb; ++s) {
        const uint32_t old = atomicCAS(&ids[s], kEmpty, want);
        if (old == kEmpty || old == want) return s;
    }
    int best = -1, bd = 0x7fffffff;
    uint32_t bb = kEmpty;
    for (int s = 0; s < kKb; ++s) {
        const uint32_t x = v[s];
        if (x == kEmpty) continue;
        const int dd = bid_distance(x, want);
        if (dd < bd) { bd = dd; best = s; bb = x; }
    }
    if (best >= 0) sel = bb;
    return best;
}

// ---------------------------------------------------------------- claim tables
// Deterministic slot claims.  A psi_out cell and an outflow bucket keep the
// first 32 distinct block ids in the order a sequential pass of the step
// claims them: the coarse (K2) batch before the fine (K3) batch; within a
// batch, a cell's own in-cell deposits (by psi_in slot, local bin, energy
// part) before the K4 transfers of faces 0..3 (by bucket slot); a bucket's
// ids by emitting column, slot, local bin, emission index.  Ids past the
// 32nd fold into the nearest kept id (smallest bid_distance, lowest slot on
// ties), as the reference's fallback does once a table is full.  The ids
// aimed at each container during one pass are gathered with their earliest
// claim key in an open-addressing row of kCand entries
// {tag << 32 | bid, (~tag) << 32 | key}; the tag is the claim pass number
// (one per transport iteration and one per injection), so entries of
// earlier passes read as free and the rows are never cleared (a wipe runs
// when the pass number nears its 32-bit limit).  Injection uses the same
// tables with the sample index as key: the reference's source kernels claim
// in sample order when run one sample at a time.  A row holds 256 ids: the
// oracle counts up to 115 distinct ids aimed at one container in one
// iteration on the reference grids and up to 181 on the 512-theta log grid;
// an id that finds no free entry is counted (cand_ovf), and a run that
// counts any is not an exact restatement of the sequential claims.
constexpr int kCandLog = 8, kCand = 1 << kCandLog;

__device__ __forceinline__ unsigned cand_hash(uint32_t bid) { return (bid * 0x9E3779B1u) >> (32 - kCandLog); }

__device__ __forceinline__ void cand_insert(unsigned long long* row, int* count, uint32_t tag, uint32_t bid,
                                            uint32_t key, int* ovf) {
    const unsigned long long tb = ((unsigned long long)tag << 32) | bid;
    const unsigned long long k = ((unsigned long long)(0xFFFFFFFFu - tag) << 32) | key;
    const unsigned h = cand_hash(bid);
    for (int p = 0; p < kCand; ++p) {
        unsigned long long* e = row + 2 * ((h + p) & (kCand - 1));
        const unsigned long long cur = __ldcg(e);
        if (cur != tb) {
            if ((uint32_t)(cur >> 32) == tag) continue;   // another id of this pass
            const unsigned long long old = atomicCAS(e, cur, tb);
            if (old == cur) atomicAdd(count, 1);
            else if (old != tb) continue;                 // taken by another id meanwhile
        }
        atomicMin(e + 1, k);
        return;
    }
    atomicAdd(ovf, 1);
}

// Slot assigned to `bid` by the selection of this pass, -1 if not gathered.
// An entry's id and slot words are read together (entries are 16-byte
// aligned), one L2 round trip per probe.
// After the selection an entry's key word holds slot | kept id << 5 (the id
// the slot holds: the entry's own, or the nearer kept id it folded into).
// RO: the tables are read-only for the rest of the kernel (the deposit
// passes), so the probes may hit in L1 (a cell's bins probe the same rows).
template <bool RO = false>
__device__ __forceinline__ int cand_find(const unsigned long long* row, uint32_t tag, uint32_t bid, uint32_t& sel) {
    const unsigned long long tb = ((unsigned long long)tag << 32) | bid;
    const unsigned h = cand_hash(bid);
    for (int p = 0; p < kCand; ++p) {
        const ulonglong2* a = reinterpret_cast<const ulonglong2*>(row + 2 * ((h + p) & (kCand - 1)));
        const ulonglong2 e = RO ? __ldg(a) : __ldcg(a);
        if (e.x == tb) {
            sel = ((uint32_t)e.y >> 5) & 0xFFFFFFu;
            return (int)((uint32_t)e.y & 31u);
        }
        if ((uint32_t)(e.x >> 32) != tag) return -1;
    }
    return -1;
}
__device__ __forceinline__ int cand_find(const unsigned long long* row, uint32_t tag, uint32_t bid) {
    uint32_t sel;
    return cand_find(row, tag, bid, sel);
}

// The first claim in cell gc puts it on occupancy list k.
__device__ __forceinline__ void mark_occupied(const Dev& d, int k, int gc) {
    if (*(volatile int*)&d.occ[k][gc] == 0 && atomicExch(&d.occ[k][gc], 1) == 0) {
        const int i = atomicAdd(&d.gs->occ_n[k], 1);
        d.occ_list[k][i] = gc;
    }
}
template <class Lay>
__device__ __forceinline__ int remap_lidx(int l, uint32_t src, uint32_t dst) {
    if (src == dst) return l;
    int t, e, x, z;
    Lay::dec(l, t, e, x, z);
    int tg = (int)(src & 0xFFFu) * Lay::NT + t;
    int eg = (int)((src >> 12) & 0xFFFu) * Lay::NE + e;
    int td = max(0, min(tg - (int)(dst & 0xFFFu) * Lay::NT, Lay::NT - 1));
    int ed = max(0, min(eg - (int)((dst >> 12) & 0xFFFu) * Lay::NE, Lay::NE - 1));
    return Lay::enc(td, ed, x, z);
}

// An entry of bkt_os: x = the value page of the psi_out slot that the
// bucket's kept id lands in (0xFFFFFFFF: none), y = the id that slot holds;
// one 8-byte load gives the fused K4 everything its resolve of a bucket id
// needs, the page included.
__device__ __forceinline__ uint2 bkt_slot_pack(int page, uint32_t sel) { return make_uint2((uint32_t)page, sel); }
__device__ __forceinline__ int bkt_slot_page(uint2 m) { return (int)m.x; }

// Value page of storage slot s of cell gc.  RO: pbase is read-only for the
// rest of the kernel (written by an earlier kernel of the pass).
template <bool RO = false>
__device__ __forceinline__ size_t page_of(const Dev& d, int gc, int s) {
    return (size_t)(RO ? __ldg(d.pbase + gc) : __ldcg(d.pbase + gc)) + (size_t)s;
}

// Phase-space value writes: the value and the bit of its float4 in the
// page's occupancy mask (a reduction whose result nobody waits for).
__device__ __forceinline__ void vmark(const Dev& d, size_t page, int lidx) {
    atomicOr(reinterpret_cast<uint32_t*>(d.vmask + page) + (lidx >> 7), 1u << ((lidx >> 2) & 31));
}
__device__ __forceinline__ void vadd(const Dev& d, size_t page, int L, int lidx, float w) {
    atomicAdd(d.val + page * (size_t)L + lidx, w);
    vmark(d, page, lidx);
}
// the float4 bits of a set of local bins, per mask word, then one
// reduction per word that received any
struct VBits {
    uint32_t w0 = 0u, w1 = 0u;
    __device__ __forceinline__ void add(int lidx) {
        const uint32_t b = 1u << ((lidx >> 2) & 31);
        if (lidx >> 7) w1 |= b;
        else w0 |= b;
    }
    __device__ __forceinline__ void flush(const Dev& d, size_t page) const {
        uint32_t* m = reinterpret_cast<uint32_t*>(d.vmask + page);
        if (w0) atomicOr(m, w0);
        if (w1) atomicOr(m + 1, w1);
    }
};

// DeviceOutflowBucket (device_bucket.cuh:48-57) with L local bins.
__host__ __device__ constexpr int bucket_bytes_for(int L) { return 32 * 4 + 32 * 2 + 32 * L * 4 + 12; }
__device__ __forceinline__ uint32_t* bucket_ids(unsigned char* b) { return reinterpret_cast<uint32_t*>(b); }
__device__ __forceinline__ float* bucket_vals(unsigned char* b) { return reinterpret_cast<float*>(b + 192); }

}  // namespace sm2d
