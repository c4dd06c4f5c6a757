// C ABI of the ILU sweep plans (senk_ilu_plan_*, senk_ilub_plan_create); the
// plans themselves are in sweep_impl.cuh, sweep_f32.cu and sweep_f64.cu.
#include <memory>

#include "device.hpp"

namespace senkgpu {
}  // namespace senkgpu

using namespace senkgpu;

extern "C" {

int senk_ilu_plan_create_sched(senk_ilu_plan **out, int dtype, int N, const void *lval, const int *lcind,
                               const int *lrptr, const void *uval, const int *ucind, const int *urptr, int precond,
                               const int *cptr, int cnum, int bsize, int sweep)
{
    return guarded("senk_ilu_plan_create", [&] {
        SENK_REQUIRE(out != nullptr, "out is null");
        auto h = std::make_unique<senk_ilu_plan>();
        h->dtype = dtype;
        if (dtype == SENK_F64) {
            h->d = std::make_unique<IluPlan<double>>();
            h->d->build(N, (const double *)lval, lcind, lrptr, (const double *)uval, ucind, urptr, precond, cptr,
                        cnum, bsize, nullptr, sweep);
        } else if (dtype == SENK_F32) {
            h->f = std::make_unique<IluPlan<float>>();
            h->f->build(N, (const float *)lval, lcind, lrptr, (const float *)uval, ucind, urptr, precond, cptr,
                        cnum, bsize, nullptr, sweep);
        } else {
            throw ArgError("dtype must be SENK_F64 or SENK_F32");
        }
        *out = h.release();
        return (int)kOk;
    });
}

int senk_ilu_plan_create(senk_ilu_plan **out, int dtype, int N, const void *lval, const int *lcind,
                         const int *lrptr, const void *uval, const int *ucind, const int *urptr, int precond,
                         const int *cptr, int cnum, int bsize)
{
    return senk_ilu_plan_create_sched(out, dtype, N, lval, lcind, lrptr, uval, ucind, urptr, precond, cptr, cnum,
                                      bsize, SENK_SWEEP_AUTO);
}

int senk_ilu_plan_status(senk_ilu_plan *plan, void *stream)
{
    return guarded("senk_ilu_plan_status", [&] {
        SENK_REQUIRE(plan, "null plan");
        (void)stream;  // the plan's sweeps report on its status word; reading it synchronises the device
        SENK_CUDA(cudaDeviceSynchronize());
        if (plan->d) plan->d->check_status(nullptr);
        else if (plan->f) plan->f->check_status(nullptr);
        return (int)kOk;
    });
}

int senk_ilu_plan_test_stall(senk_ilu_plan *plan, int upper, int group)
{
    return guarded("senk_ilu_plan_test_stall", [&] {
        SENK_REQUIRE(plan && (plan->d || plan->f), "null plan or not a CSR factor plan");
        auto stall = [&](auto &P) {
            auto &F = upper ? P.U : P.L;
            if (F.persistent) {
                bool barrier = false;
                for (const auto &L : F.launches) barrier = barrier || (L.coop && L.cend - L.cbeg >= 2);
                SENK_REQUIRE(barrier, "the sweep has no cooperative launch with a grid barrier");
                // arrivals start far below any barrier's target
                const int low = -(1 << 30);
                SENK_CUDA(cudaMemcpy(F.ctrl.p, &low, sizeof(int), cudaMemcpyHostToDevice));
                return;
            }
            SENK_REQUIRE(F.dataflow, "the factor is not swept by the dataflow or cooperative schedule");
            SENK_REQUIRE(group >= 0 && group < F.ngroups, "group out of range");
            int ptr[2];
            SENK_CUDA(cudaMemcpy(ptr, F.dep_ptr.p + group, sizeof(ptr), cudaMemcpyDeviceToHost));
            SENK_REQUIRE(ptr[1] > ptr[0], "the group reads from no other group");
            // the group's first dependency becomes the group itself, whose flag
            // cannot be set before the group has run
            SENK_CUDA(cudaMemcpy(F.dep_idx.p + ptr[0], &group, sizeof(int), cudaMemcpyHostToDevice));
        };
        if (plan->d) stall(*plan->d);
        else stall(*plan->f);
        return (int)kOk;
    });
}

int senk_ilub_plan_create(senk_ilu_plan **out, int N, int bnl, int bnw, const double *blval, const int *blcind,
                          const int *blrptr, const double *buval, const int *bucind, const int *burptr,
                          const int *cptr, int cnum, int bsize)
{
    return guarded("senk_ilub_plan_create", [&] {
        SENK_REQUIRE(out != nullptr, "out is null");
        auto h = std::make_unique<senk_ilu_plan>();
        h->dtype = SENK_F64;
        h->b = std::make_unique<IlubPlan<double>>();
        h->b->build(N, bnl, bnw, blval, blcind, blrptr, buval, bucind, burptr, cptr, cnum, bsize, nullptr);
        *out = h.release();
        return (int)kOk;
    });
}

int senk_ilu_plan_apply(senk_ilu_plan *plan, const void *x, void *y, void *stream)
{
    return guarded("senk_ilu_plan_apply", [&] {
        SENK_REQUIRE(plan && x && y, "null argument");
        cudaStream_t s = (cudaStream_t)stream;
        if (plan->b) plan->b->apply((const double *)x, (double *)y, s, nullptr);
        else if (plan->d) plan->d->apply((const double *)x, (double *)y, s, nullptr);
        else plan->f->apply((const float *)x, (float *)y, s, nullptr);
        SENK_LAUNCH_CHECK();
        return (int)kOk;
    });
}

int senk_ilu_plan_sweep(senk_ilu_plan *plan, int upper, const void *x, void *y, void *stream)
{
    return guarded("senk_ilu_plan_sweep", [&] {
        SENK_REQUIRE(plan && x && y, "null argument");
        cudaStream_t s = (cudaStream_t)stream;
        if (plan->b) plan->b->sweep(upper != 0, (const double *)x, (double *)y, s, nullptr);
        else if (plan->d) plan->d->sweep(upper ? plan->d->U : plan->d->L, (const double *)x, (double *)y, s, nullptr);
        else plan->f->sweep(upper ? plan->f->U : plan->f->L, (const float *)x, (float *)y, s, nullptr);
        return (int)kOk;
    });
}

int senk_ilu_plan_destroy(senk_ilu_plan *plan)
{
    return guarded("senk_ilu_plan_destroy", [&] {
        delete plan;
        return (int)kOk;
    });
}

}  // extern "C"
