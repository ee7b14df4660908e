function data = fwd_PDE_exact_MNAD(dx,xs,xr,dz,zs,zr,v,dt,nt,w,d_pml,ss,Auu,Auv,Auw,Avu,Avv,Avw,Awu,Awv,Aww,indx)
% GB300 drop-in for SRC/MNAD/fwd_PDE_exact_MNAD.m (same arguments, same
% return value data = {datau}).  The nine operators are recomputed on the
% GPU from v, dx, dz, dt and are ignored here.  With indx == 1 the d2u
% snapshots and the illumination stay on the GPU under shot id ss; they are
% also written to ./Wavefields/UU_<ss>.mat and ./Illuminations/illum_<ss>.mat
% (as the reference does) when MNAD_WRITE_WAVEFIELDS is set, for drivers
% whose forward and adjoint of one shot run in different parfor workers.
if nargin < 22 || isempty(indx)
    indx = 0;
end
data = mnad_mex('fwd', dx, xs, xr, dz, zs, zr, v, dt, nt, w, d_pml, ss, indx);
if indx == 1 && ~isempty(getenv('MNAD_WRITE_WAVEFIELDS'))
    [UU, illum] = mnad_mex('export', ss);
    illum = reshape(illum, size(v,1) - 2*d_pml, size(v,2) - 2*d_pml);
    if ~exist('./Wavefields', 'dir'), mkdir('./Wavefields'); end
    if ~exist('./Illuminations', 'dir'), mkdir('./Illuminations'); end
    save(['./Wavefields/UU_' num2str(ss) '.mat'], 'UU');
    save(['./Illuminations/illum_' num2str(ss) '.mat'], 'illum');
end
end
