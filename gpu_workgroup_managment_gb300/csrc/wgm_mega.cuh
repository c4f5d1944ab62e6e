/*
 * The megakernel's built-in persistent apps: the argument block wgm_k_mega
 * (csrc/wgm_mega.cu) takes.  The runtime the megakernel runs on - the
 * scheduler, offer_kill / offer_fork, the resizing barrier, the worker loop
 * (wgm_mega_body) and the non-persistent tasks - is in include/wgm_device.cuh,
 * where apps built outside the library use the same code.
 */
#ifndef WGM_MEGA_CUH
#define WGM_MEGA_CUH

#include "wgm_graph.cuh"
#include "wgm_octree.cuh"
#include "wgm_c4.cuh"

/* Persistent app hosted by the megakernel: `app` selects which of the
 * argument blocks is used; ctl is the control block of every megakernel. */
struct wgm_mega_args {
  int app; /* WGM_K_* of the persistent app, -1: none */
  wgm_lonestar_args ls;
  wgm_color_args color;
  wgm_mis_args mis;
  wgm_psssp_args psssp;
  wgm_pr_args pr;
  wgm_bc_args bc;
  wgm_octree_args oct;
  wgm_c4_args c4;
  wgm_mega_ctl ctl;
};

#endif
