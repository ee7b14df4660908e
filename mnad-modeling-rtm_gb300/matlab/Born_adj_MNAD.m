function Im = Born_adj_MNAD(dx,dz,nt,dt,v,xr,zr,data,d_pml,ss,Auu,Auv,Auw,Avu,Avv,Avw,Awu,Awv,Aww)
% GB300 drop-in for SRC/migration/Born_adj_MNAD.m (same arguments, Im is
% Nint x 1).  data may be the cell {datau} or the nt x nr matrix.  The source
% wavefield of shot ss is the one the forward kept on the GPU of this MATLAB
% process; when this process does not hold it (parfor placed the forward in
% another worker), it is loaded from ./Wavefields/UU_<ss>.mat as the
% reference does (Born_adj_MNAD.m:33).
if ~mnad_mex('has', ss)
    S = load(['./Wavefields/UU_' num2str(ss) '.mat']);
    nf = floor(nt/(2*3*max(v(:))/min(v(:))));
    T = floor(nt/nf/2);
    mnad_mex('import', ss, size(v,1), size(v,2), d_pml, nt, T, S.UU);
end
Im = mnad_mex('adj', dx, dz, nt, dt, v, xr, zr, data, d_pml, ss);
mnad_mex('release', ss);
end
