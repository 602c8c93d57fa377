/* nmesh_nmgdump.h -- declarations of the dump add-on module (test-side) */
int nmgdump_perturb(tMesh *mesh);
int nmgdump_rhs(tMesh *mesh);
int nmgdump_final(tMesh *mesh);
