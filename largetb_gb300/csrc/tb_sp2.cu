// tb_sp2.cu -- SP2 block SpGEMM kernels (in progress)
