// One kernel variant. The build compiles this file once per entry of gqs_variant_table.h,
// with -DGQS_TU_LIST=GQS_VARIANTS_<TYPE> -DGQS_TU_TYPE=<type> -DGQS_TU_INDEX=<index>, so the
// variants build in parallel and each object holds exactly one kernel configuration.
#include "gqs_variant_table.h"
#include "gqs_variants.cuh"

#if !defined(GQS_TU_LIST) || !defined(GQS_TU_TYPE) || !defined(GQS_TU_INDEX)
#error "compile with -DGQS_TU_LIST=... -DGQS_TU_TYPE=... -DGQS_TU_INDEX=..."
#endif

#define GQS_PP_CAT_(a, b) a##b
#define GQS_PP_CAT(a, b) GQS_PP_CAT_(a, b)
#define GQS_FN(base) GQS_PP_CAT(GQS_PP_CAT(base, GQS_TU_TYPE), GQS_PP_CAT(_, GQS_TU_INDEX))

namespace gqs {
namespace {
template <int I>
struct Pick;
#define GQS_PICK(S, V, T, NCW, TILE, CHUNK, STAGES, R)                                \
  template <>                                                                         \
  struct Pick<V> {                                                                    \
    using C = Cfg<T, NCW, TILE, CHUNK, STAGES, R>;                                    \
    static const char* name() { return #S "_ncw" #NCW "_tile" #TILE "_chunk" #CHUNK "_st" #STAGES; } \
  };
GQS_TU_LIST(GQS_PICK)
#undef GQS_PICK
using Chosen = Pick<GQS_TU_INDEX>;
}  // namespace

VariantInfo GQS_FN(info_)() { return VariantOps<Chosen::C>::info(Chosen::name()); }
int GQS_FN(prepare_)() { return VariantOps<Chosen::C>::prepare(); }
cudaError_t GQS_FN(launch_)(const LaunchParams& p) { return VariantOps<Chosen::C>::launch(p); }

}  // namespace gqs
