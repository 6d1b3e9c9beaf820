/*
 * jlgs_driver.c -- test-only shim that drives the reference's own
 * gather-scatter library (NekCEM src/jl/gs.c, compiled from the reference
 * tree by oracle/build_ref.sh into oracle/_ref/libjlgs.so).
 *
 * It performs exactly the call sequence of the Fortran side:
 *   gs_setup(gsh_face, glo_num, ntot, nekcomm, np)     src/nek5_connect11.F:2223
 *   gs_op_fields(gsh_face, srflx, nxzfl, 6, 1, 1, 0)     src/cem_maxwell.F:962
 *   gs_free(gsh_face)
 * on a single process (no MPI), so tests can compare the oracle's face
 * exchange against the reference implementation on the same ids and data.
 */
typedef int sint_t;
typedef long long slong_t;

void gs_setup_(sint_t* handle, const slong_t* id, const sint_t* n, const int* comm,
               const sint_t* np);
void gs_op_fields_(const sint_t* handle, void* u, const sint_t* stride, const sint_t* n,
                   const sint_t* dom, const sint_t* op, const sint_t* transpose);
void gs_free_(const sint_t* handle);

/* tensor.c is linked only for tensor_dot (used by comm.c); nothing on the gs path calls mxm */

int jlgs_apply(const long long* ids, int n, double* u, int stride, int nfld) {
  sint_t h = -1, nn = n, np = 1, st = stride, nf = nfld, dom = 1, op = 1, tr = 0;
  int comm = 0;
  if (n <= 0 || stride < n || nfld < 1) return -1;
  gs_setup_(&h, (const slong_t*)ids, &nn, &comm, &np);
  if (h < 0) return -2;
  gs_op_fields_(&h, u, &st, &nf, &dom, &op, &tr);
  gs_free_(&h);
  return 0;
}
