/* geo_stub.c -- link stubs for the two geogram symbols that global_types.cpp of the reference
 * references through its unused global `GEO::Mesh M_i` (constructor and destructor).  The
 * hot-path functions never touch that object, so the stubs do nothing.  Used only for the
 * oracle/_ref build.  TEST INFRASTRUCTURE ONLY. */
void _ZN3GEO4MeshC1Ejb(void *self, unsigned int dim, _Bool single_precision) {
  (void)self; (void)dim; (void)single_precision;
}
void _ZN3GEO4MeshD1Ev(void *self) { (void)self; }
