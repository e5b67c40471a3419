// tb_dos.cu -- stochastic KPM DOS kernels (in progress)
