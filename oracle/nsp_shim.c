/*
 * Interposed symbols for the -nsp build of the reference (oracle/_ref/skid_nsp,
 * made by oracle/build_ref.sh).  Test infrastructure only.
 *
 * -nsp ("no scatterer pruning") is described in the reference's README but
 * v1.4.1 does not implement it.  The patched oracle keeps every scatterer:
 *  - ScatterCut (smooth1.c:387-405) partitions the scatterers by density
 *    and returns how many stay; this one keeps all n.  smooth1.c is built as
 *    a shared object, so its own call goes through the PLT and binds to the
 *    executable's definition here.
 *  - main.c asks bAllowInitialCut (kd.c:696-699) whether the first step may
 *    zero the untouched scatterers' densities (main.c:396-401); main.c is
 *    compiled with that name mapped to nsp_no_initial_cut, which says no.
 * Pointer arguments are declared void *: only the ABI matters here.
 */
int ScatterCut(void *p, int n, float fScatDens)
{
    (void)p;
    (void)fScatDens;
    return n;
}

int nsp_no_initial_cut(void *kd)
{
    (void)kd;
    return 0;
}
