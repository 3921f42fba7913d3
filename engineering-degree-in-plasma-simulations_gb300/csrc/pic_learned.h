// Learned multilevel Poisson preconditioner: level views, parameters and launch functions.
//
// B r = mask * sum_l P^l o_l over a hierarchy of boxes (level 0 = the distinct nodes of the
// grid, level l+1 = level l halved per axis, rounding up), with cell-centred trilinear
// prolongation P and its transpose R as restriction.  Level 0 applies a learned 3x3x3
// stencil, levels 1..4 a linear convolutional network (3x3x3 lift 1 -> C, C x C channel mix,
// 3x3x3 projection C -> 1; C = 16, 32, 64, 64), deeper levels the inverse Galerkin diagonal.
// Inference folds each network level into an exact 5x5x5 stencil; training runs the network
// unfolded, its contractions on the tensor cores (tcgen05, BF16 operands, FP32 accumulators).
#pragma once
#include <cuda_bf16.h>
#include "pic_kernels.h"

namespace pic {

constexpr int kLpMaxLevels = 12;
constexpr int kLpNetLevels = 4;
__host__ __device__ constexpr int lp_channels(int l) { return l == 1 ? 16 : l == 2 ? 32 : 64; }

// a 3-D box of FP32 values: element (x, y, z) at a[x + y*sy + z*sz]
struct LView {
    float* a;
    int n[3];
    int sy, sz;
    int per[3];
    FastDiv fx, fxy;  // decode of a linear voxel index (x fastest)
    int nvox;
};

// offsets of the parameter groups inside the flat FP32 parameter array
struct LpLayout {
    int total;
    int s0;                       // level-0 stencil, 27
    int wl[kLpNetLevels + 1];     // lift  [C][27]
    int wm[kLpNetLevels + 1];     // mix   [C][C] (out, in)
    int wp[kLpNetLevels + 1];     // proj  [27][C]
};
constexpr int kLpFold = 729 + 125;  // per network level: K27 [27][27] then K5 [125] (staged in shared memory)
// then the 27 face-class variants of K5 [27][125] (class cx + 3 cy + 9 cz per axis: 0 away from a
// non-periodic face, 1 on its low face, 2 on its high face; variant 0 is K5)
constexpr int kLpFoldStride = kLpFold + 27 * 125;

struct LpTrain;

struct LpState {
    int nlev = 0;
    int dims[kLpMaxLevels][3] = {};
    int per[3] = {0, 0, 0};
    double diag[kLpMaxLevels] = {};
    float* z[kLpMaxLevels] = {};  // restricted input, levels >= 1
    float* e[kLpMaxLevels] = {};  // level output, levels >= 1
    LpLayout lay{};
    float* W = nullptr;     // parameters (FP32 master copy)
    float* fold = nullptr;  // folded stencils, kLpFoldStride per network level (index l-1)
    LpTrain* train = nullptr;
    // host copy of every network level's K5, passed to the tiled level kernel as a parameter
    // (the constant bank feeds the FMAs directly); refreshed on the first apply after a fold
    mutable float k5_host[kLpNetLevels][125] = {};
    mutable bool k5_valid = false;
};

LView lp_view(float* a, const int n[3], int sy, int sz, const int per[3]);
LView lp_level_view(const LpState& L, int l, float* a);
LView lp_node_view(const GridDev& g, const LpState& L, float* a);  // level 0 over the node array

void lp_layout(LpLayout& lay);
void lp_init_weights(const LpLayout& lay, const double* diag, int nlev, float* host_W);
void lp_galerkin_diag(const double c[3], int nlev, double* diag);

void launch_lp_fold(const LpState& L, cudaStream_t s);
void lp_free_train(LpState& L);
// training (see pic_learned.cu): allocation, bf16 operand copies, one loss + gradient evaluation,
// a white-noise sample pair, one Adam step (followed by the bf16 copies and the folds)
int lp_alloc_train(const GridDev& g, LpState& L, const float* init_W);
void launch_lp_prep(const LpState& L, cudaStream_t s);
void launch_lp_loss_grad(const GridDev& g, LpState& L, const uint16_t* kind, const float* r, const float* x,
                         cudaStream_t s, int grid, int sms);
void launch_lp_noise_pair(const GridDev& g, LpState& L, const uint16_t* kind, unsigned long long seed, cudaStream_t s,
                          int grid);
void launch_lp_adam(LpState& L, float lr, cudaStream_t s);
int lp_pair_begin(LpState& L, const float* r0, int nv, cudaStream_t s);
void lp_pair_add(LpState& L, const float* e, int nv, cudaStream_t s, int grid);
void lp_pair_end(LpState& L);
const float* lp_pair_r(const LpState& L, int k);
const float* lp_pair_x(const LpState& L, int k);
int lp_npairs(const LpState& L);
// first-wait poll count of the tensor-core kernels (PushArgs::wait_polls convention; test hook)
int lp_set_tc_wait_polls(long long arg);
float* lp_train_x(const LpState& L);
float* lp_train_val(const LpState& L);
float* lp_train_wprev(const LpState& L);
float* lp_train_r(const LpState& L);
float* lp_train_grad(const LpState& L);
double* lp_train_red(const LpState& L);
unsigned* lp_train_err(const LpState& L);
// z = B r on the node array (r zero off FREE nodes); with red != nullptr the last kernel also
// sums z.r and z.q into red->scal[kS_RZN], [kS_RZO]; every kernel returns early when flag[0] is
// set (inner solve converged)
void launch_lp_apply(const GridDev& g, const LpState& L, const float* r, float* z, const uint16_t* kind,
                     const float* q, const SolveWork* red, const int* flag, cudaStream_t s, int sms);
// flexible CG iteration with the learned preconditioner (see pic_learned.cu)
void launch_lp_norm2(const float* a, int n, double* part, double* out, cudaStream_t s, int grid);
void launch_lpcg_init(const GridDev& g, SolveWork& w, const LpState& L, cudaStream_t s, int sms);
void launch_lpcg_iter(const GridDev& g, SolveWork& w, const LpState& L, float* d_in, float* d_out, int it,
                      double target_rr, cudaStream_t s, int sms);
void launch_lpcg_k1_probe(const GridDev& g, SolveWork& w, float* d_in, float* d_out, cudaStream_t s);

}  // namespace pic
