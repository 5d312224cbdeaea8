// Device state of the ALI level-population loop (mgr_ali.cu).
#pragma once
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
    double phase_ms[4] = {0.0, 0.0, 0.0, 0.0};
};

// Jlin: the memory-lean solve's line-integrated J [P][L] (compute_Jeff_sparse), or NULL.
cudaError_t ali_launch_jeff(MgrModel* model, const double* J, const double* lam, const double* Jlin = nullptr);
// Drops the captured iteration after the ray-pair shard or its reduce function changed.
void ali_shard_changed(MgrModel* model);
cudaError_t ali_launch_stateq_and_refresh(MgrModel* model, const double* lam);
cudaError_t ali_launch_line_refresh(MgrModel* model);
cudaError_t ali_ng_step(MgrModel* model, int order);
cudaError_t ali_ng_trial(MgrModel* model, int order);
cudaError_t ali_history_push_all(MgrModel* model);
void ali_free(MgrModel* model);

}  // namespace mgr
