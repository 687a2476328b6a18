// ao2mo_split.cu -- placeholder until the tcgen05 split-precision path lands.
#include "internal.h"
namespace mq {
int ao2mo_split_device(mq_ctx *c, const double *, int, const double *, int, const double *, int, const double *, int,
                       double *) {
  return set_err(c, MQ_EINVAL, "split-precision transform not built");
}
}  // namespace mq
