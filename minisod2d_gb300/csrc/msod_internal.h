// msod_internal.h -- shared host-side helpers of the msod library (not part of the ABI).
#pragma once

#include <cstdarg>
#include <cstdint>
#include <cstdio>

#include "msod.h"

namespace msod {

// Records `code` with a printf-style message as the calling thread's last
// error and returns `code`.
int set_error(int code, const char *fmt, ...);
// Clears the calling thread's last error.
void clear_error();
// Whether checked mode is on (validation + synchronisation in every call).
bool checked_mode();

// The form chosen by msod_set_mode (msod_mode.cu).
bool mode_is_default_convec();
bool mode_is_default_diffusion();
void mode_release();
int mode_convec(int porder, int nelem, int npoin, const int *connec, const float *He, const float *gpvol,
                const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                const int *gmshAtoK, const float *u, const float *q, const float *rho, const float *pr,
                const float *E, float *Rmass, float *Rmom, float *Rener, void *stream);
int mode_diffusion(int porder, int nelem, int npoin, const int *connec, const float *He, const float *gpvol,
                   const float *dlxigp_ip, const int *invAtoIJK, const int *gmshAtoI, const int *gmshAtoJ,
                   const int *gmshAtoK, float Cp, float Pr, const float *rho, const float *u, const float *Tem,
                   const float *mu_fluid, const float *mu_e, const float *mu_sgs, float *Rmass, float *Rmom,
                   float *Rener, void *stream);

}  // namespace msod
