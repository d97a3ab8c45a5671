/*
 * Field injection for the reference build. TEST INFRASTRUCTURE ONLY.
 *
 * The reference finder smooths its grid once per rung and reads the result
 * back through sif__fft_grid_backward() (src/math/fft.c:820-888; called from
 * src/finder/exodus_finder.c:1723-1727 and the restore at 2432-2453). The
 * strict reference library is linked with -Wl,--wrap of that symbol, so every
 * such call lands here first. Unarmed, this passes straight through.
 *
 * Armed with orc_hook_inject(), the k-th call's output is overwritten with the
 * k-th injected field (k below the count given); later calls, such as the
 * grid restore at the end of the run, pass through. This lets the reference's
 * own candidate scan, sort, rescaling and overlap cleaning run on exactly the
 * smoothed fields another implementation saw, which is how catalogue identity
 * is tested independently of FFT rounding.
 *
 * orc_hook_capture() records the fields the reference itself produced.
 */
#include <stdint.h>
#include <string.h>

typedef struct sif_fft_workspace sif_fft_workspace_t;

/* The reference's sif_real: the fields are in the precision it was built in. */
#ifdef SIF_USE_DOUBLE
typedef double hook_real;
#else
typedef float hook_real;
#endif

hook_real* __real_sif__fft_grid_backward(sif_fft_workspace_t* ws);

static const hook_real* g_inject;
static hook_real* g_capture;
static uint64_t g_cells;
static uint32_t g_n_inject, g_n_capture, g_calls;

void orc_hook_inject(const hook_real* fields, uint64_t cells, uint32_t n_fields) {
  g_inject = fields;
  g_cells = cells;
  g_n_inject = fields ? n_fields : 0;
  g_calls = 0;
}

void orc_hook_capture(hook_real* out, uint64_t cells, uint32_t n_max) {
  g_capture = out;
  g_cells = cells;
  g_n_capture = out ? n_max : 0;
  g_calls = 0;
}

uint32_t orc_hook_calls(void) { return g_calls; }

hook_real* __wrap_sif__fft_grid_backward(sif_fft_workspace_t* ws) {
  hook_real* r = __real_sif__fft_grid_backward(ws);
  if (r) {
    if (g_capture && g_calls < g_n_capture)
      memcpy(g_capture + (uint64_t)g_calls * g_cells, r, g_cells * sizeof(hook_real));
    if (g_inject && g_calls < g_n_inject)
      memcpy(r, g_inject + (uint64_t)g_calls * g_cells, g_cells * sizeof(hook_real));
  }
  g_calls++;
  return r;
}
