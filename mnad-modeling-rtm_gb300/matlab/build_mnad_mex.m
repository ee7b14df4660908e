function build_mnad_mex(repo)
% Builds the MEX gateway against libmnad.so of the GB300 MNAD library.
% repo: the repository root (containing include/ and mnad-modeling-rtm_gb300/).
libdir = fullfile(repo, 'mnad-modeling-rtm_gb300', 'mnad', '_lib');
here = fileparts(mfilename('fullpath'));
mex('-R2017b', fullfile(here, 'mnad_mex.c'), ['-I' fullfile(repo, 'include')], ['-L' libdir], '-lmnad', ...
    ['LDFLAGS=$LDFLAGS -Wl,-rpath,' libdir], '-outdir', here);
end
