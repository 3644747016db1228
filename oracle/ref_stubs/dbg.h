/* The dbg-macro submodule is empty in the reference checkout; the reference
 * only includes the header and never calls dbg(). */
#pragma once
