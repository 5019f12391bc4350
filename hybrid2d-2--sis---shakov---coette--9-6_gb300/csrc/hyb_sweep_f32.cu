// hyb_sweep_f32.cu -- FP32-distribution instantiations of the fused sweep.
#include "hyb_sweep.cuh"
#include "hyb_sweep_nnd.cuh"

namespace hyb {
int sweep_launch_f32(hyb_ctx *ctx, const KinArgs<float> &A, int cpt, int vpb, bool launch) {
    if (sweep_nnd_ok(ctx, cpt)) return sweep_nnd_dispatch(ctx, A, vpb, launch);
    return sweep_launch_real<float>(ctx, A, cpt, vpb, launch);
}
size_t sweep_nnd_group_bytes_f32(int PA, int tpv) { return nnd_group_bytes(PA, tpv); }
int sweep_nnd_batch_f32(const KinArgs<float> *args, const int2 *work, int nwork, int PA, int vpb, int sig,
                        cudaStream_t s) {
    return sweep_nnd_batch(args, work, nwork, PA, vpb, sig, s);
}
size_t sweep_group_bytes_f32(int PA, int tpv) { return sweep_group_bytes<float>(PA, tpv); }
int sweep_batch_f32(const KinArgs<float> *args, const int2 *work, int nwork, int PA, int cpt, int vpb, bool uni,
                   int scheme, cudaStream_t s) {
    return sweep_batch_real<float>(args, work, nwork, PA, cpt, vpb, uni, scheme, s);
}
}  // namespace hyb
