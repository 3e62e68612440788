/* The reference's NEON and SME backends are AArch64 Mach-O assembly and are not built here.
 * These stand-ins refuse to initialise, so an explicit neon/sme request fails and AUTO falls
 * back to the reference's portable `ref` backend.  Test infrastructure only. */
#include "internal.h"

static int refshim_no_init(kite_ctx *ctx) { (void)ctx; return -1; }

const kite_backend_ops kite_neon_ops = {.name = "neon (not built)", .init = refshim_no_init};
const kite_backend_ops kite_sme_ops = {.name = "sme (not built)", .init = refshim_no_init};
