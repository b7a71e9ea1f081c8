/* d3b2_create_matrix: single-object assembly and inverse on the GPU.
 * Usage (as the reference's tool): medium_file mesh_file output.obj [rv_x rv_y rv_z theta tr_x tr_y tr_z] */
#include "bem3_emf_b2.h"

int main(int argc,char **argv)
{
  DOMD md;
  read_domd2(argc,argv,&md);
  print_domd2(&md);
  initialize_domd2(&md);
  create_matrix(&md,argv[3]);
  finalize_domd2(&md);
  return 0;
}
