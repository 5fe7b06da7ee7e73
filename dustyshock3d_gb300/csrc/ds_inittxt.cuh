// Init.txt readers behind ds_params_read_init_txt and ds_ic_read_init_txt.
#pragma once

#include "../../include/dustyshock3d_gb300.h"

// The 17 positional values (kernel.cu:1705-1723) into p, then the extension
// lines "name = value" after line 18 ("ic" lines skipped).  DS_ERR_ARG for a
// missing file, a malformed value or an unknown name.
ds_status ds_read_init_txt_file(const char *path, ds_params *p);

// The "ic = <kind>" and "ic.<field> = value" extension lines (no "ic" line:
// DS_IC_SOD_X_DUST, the reference's generator).
ds_status ds_read_ic_txt_file(const char *path, ds_ic *ic);
