// hyb_sweep_f64.cu -- FP64-distribution instantiations of the fused sweep.
#include "hyb_sweep.cuh"

namespace hyb {
int sweep_launch_f64(hyb_ctx *ctx, const KinArgs<double> &A, int cpt, int vpb, bool launch) {
    return sweep_launch_real<double>(ctx, A, cpt, vpb, launch);
}
size_t sweep_group_bytes_f64(int PA, int tpv) { return sweep_group_bytes<double>(PA, tpv); }
int sweep_batch_f64(const KinArgs<double> *args, const int2 *work, int nwork, int PA, int cpt, int vpb, bool uni,
                   int scheme, cudaStream_t s) {
    return sweep_batch_real<double>(args, work, nwork, PA, cpt, vpb, uni, scheme, s);
}
}  // namespace hyb
