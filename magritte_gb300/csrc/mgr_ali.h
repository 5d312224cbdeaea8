// Device state of the ALI level-population loop (mgr_ali.cu).
#pragma once
#include <string>
#include <vector>

#include "mgr_internal.h"

namespace mgr {

constexpr int kMaxNgOrder = 16;   // largest Ng acceleration order (Ng_acceleration_mem_limit)
constexpr int kMaxLevels = 64;    // levels per species (shared-memory rate block, level masks)
constexpr int kConvBlocks = 256;  // blocks of the convergence reduction
constexpr int kGramBlocks = 256;  // blocks of the Ng Gram-matrix reduction

// One collision partner on the device (collisionPartner.hpp).
struct ColParView {
    uint32_t num;        // abundance column of the partner
    int32_t ortho_para;  // 0 'n', 1 'o', 2 'p'
    uint32_t ncol, ntmp;
    const uint32_t* icol;
    const uint32_t* jcol;
    const double* tmp;
    const double* Cd;  // [ntmp][ncol]
    const double* Ce;
};

// One line-producing species, passed by value to the kernels.
struct SpeciesView {
    uint32_t num, nlev, nrad, line_offset, ncolpar;
    uint32_t ncol_total;   // collisional transitions summed over the partners
    const double* energy;
    const double* weight;
    const uint32_t* irad;  // upper level
    const uint32_t* jrad;  // lower level
    const double* A;
    const double* Bs;
    const double* Ba;
    const double* freq;
    const ColParView* cp;  // [ncolpar], device
    double* pop;           // [P][nlev] FP64
    const double* tot;     // [P] population_tot
    double* Jlin;          // [P][nrad]
    double* Jeff;
    double* Jdif;
};

// Up to kMaxNgOrder device vectors, passed by value (graph-friendly).
struct VecList {
    const double* v[kMaxNgOrder];
};

struct AliSpecies {
    SpeciesView view{};
    double* prev1 = nullptr;       // population_prev1
    double* trial = nullptr;       // trial_population
    double* trial_prev = nullptr;  // trial_population_prev
    std::vector<double*> hist;     // populations list (oldest first)
    std::vector<double*> res;      // residuals list (oldest first)
    std::vector<double*> free_bufs;
    double* take_buffer();
    void clear_residuals();
    void keep_last_population();
    void pop_back_history();
};

// The global rate system (n_off_diag > 0): per point block an LU factorisation (the
// block-Jacobi preconditioner), and over all points BiCGSTAB on the preconditioned,
// population-scaled operator.  The band elements couple point p's lower level to the
// upper level of the element's point nr; the diagonal term they add to nr's own block
// is gathered through a CSR of the elements by (nr, upper level), built once per ALI
// call (the rays, hence the elements' points, do not change between iterations).
struct GlobalRate {
    bool built = false;                 // CSR of the current ALI call
    std::vector<uint32_t*> csr_off;     // per species: [P nlev + 1] row starts
    std::vector<uint32_t*> csr_ent;     // per species: element indices (into coef), ascending per row
    std::vector<size_t> csr_cap;        // entries allocated per species
    uint32_t* cursor = nullptr;         // [P max_nlev + 1] counts, then fill cursors
    double* lu = nullptr;               // [P][nlev^2] LU factors of the point blocks
    uint32_t* piv = nullptr;            // [P][nlev] row interchanges
    double* coef = nullptr;             // [P][nrad][hnrays 2K] v of each band element
    double* vec = nullptr;              // 9 vectors of P nlev (x, r, rhat, p, v, s, t, rhs, spare)
    double* red = nullptr;              // reduction partials [kConvBlocks] and results [8]
    double* red_host = nullptr;         // pinned copy of the results
    size_t cap_n = 0, cap_lu = 0, cap_coef = 0;
    int last_iterations = 0;            // BiCGSTAB iterations of the latest solve
    double last_residual = 0.0;         // its final max-norm residual relative to the right-hand side
    std::vector<void*> allocs;
};

struct AliState {
    std::vector<AliSpecies> species;
    std::vector<void*> allocs;       // every device allocation of this state
    std::vector<void*> pool_allocs;  // history buffer pool
    const double* abundance = nullptr;  // [P][nspecs] device
    uint32_t nspecs = 0;
    MgrAliParams prm{};
    bool keep_history = false;
    double* partial = nullptr;       // convergence partials [kConvBlocks][3]
    double* stats_dev = nullptr;     // [nlspecs][3] fraction_not_converged, mean, max
    double* stats_host = nullptr;    // pinned copy
    double* gram_partial = nullptr;  // [kGramBlocks][kMaxNgOrder^2]
    double* coef = nullptr;          // [kMaxNgOrder]
    size_t pool_per_species = 0;
    cudaGraphExec_t graph = nullptr;
    int graph_precision = -1;
    bool graph_failed = false;
    bool reduce_failed = false;  // the ray-shard reduce function returned an error
    // memory-lean variant (compute_level_populations_sparse): line-integrated J per
    // iteration instead of J per frequency
    bool sparse = false;
    int graph_sparse = -1;
    double* Jlin_buf = nullptr;  // [P][L]
    size_t Jlin_bytes = 0;
    // Per-phase device time of the last compute_level_populations: events between the
    // phases of a normal iteration (recorded inside the captured graph) and around the
    // Ng steps; ms of [formal solve (and shard reduce), Jeff, statistical equilibrium
    // with corrections / convergence / line-data refresh, Ng steps].
    cudaEvent_t ev[6] = {};
    bool timing = false;
    std::string timing_error;  // why the phase timing stopped, when it did
    double phase_ms[4] = {0.0, 0.0, 0.0, 0.0};
    // Non-local ALO (n_off_diag > 0): the band elements of the latest formal solve
    // [P][L][hnrays][2 n_off_diag] (the model's alo_scratch / alo_nr_scratch, which
    // outlive this state for mgr_compute_jeff) and the global rate system.
    double* alo_off = nullptr;
    uint32_t* alo_nr = nullptr;
    GlobalRate grs;
};

// Jlin: the memory-lean solve's line-integrated J [P][L] (compute_Jeff_sparse), or NULL.
// alo_off / alo_nr: the band elements of the same formal solve (n_off_diag > 0), or NULL.
cudaError_t ali_launch_jeff(MgrModel* model, const double* J, const double* lam, const double* Jlin = nullptr,
                            const double* alo_off = nullptr, const uint32_t* alo_nr = nullptr);
// Drops the captured iteration after the ray-pair shard or its reduce function changed.
void ali_shard_changed(MgrModel* model);
cudaError_t ali_launch_stateq_and_refresh(MgrModel* model, const double* lam);
cudaError_t ali_launch_line_refresh(MgrModel* model);
cudaError_t ali_ng_step(MgrModel* model, int order);
cudaError_t ali_ng_trial(MgrModel* model, int order);
cudaError_t ali_history_push_all(MgrModel* model);
void ali_free(MgrModel* model);

}  // namespace mgr
