classdef bemretgpu < bembase
  %  BEMRETGPU - Retarded BEM solver on the GPU (drop-in for BEMRET).
  %    Same calling surface as BEMRET (BEM/@bemret):
  %      bem = bemsolver( p, op );          %  op.sim = 'ret', op.gpu set
  %      sig = bem \ exc( p, enei );        %  compstruct with sig1, sig2, h1, h2
  %      ext = exc.ext( sig );  sca = exc.sca( sig );
  %    The assembly of G1, H1, G2, H2, the block LDU factorisations, the
  %    mldivide chain and the refinement run in libmnpbem_gpu through the MEX
  %    gateway mnpbem_gpu_mex.  BEMSOLVER picks this class over BEMRET because
  %    it meets one more need (Base/@bembase/find.m counts the agreements).
  %
  %    Options read from OP: RelCutoff, AbsCutoff, order (as bemoptions),
  %    device (CUDA ordinal, default 0), precision ('mixed' default, or
  %    'fp64'), refine_tol (default 1e-10).  Flat boundary elements only in
  %    this class (p.interp = 'flat'); nested media are not supported.

  properties (Constant)
    name = 'bemsolver'
    needs = { struct( 'sim', 'ret' ), 'gpu' }
  end

  properties
    p                       %  compound of discretized particles
    enei = []               %  wavelength of the last solve
    precision = 'mixed'     %  'mixed' (complex64 TF32 + refinement) or 'fp64'
    refine_tol = 1e-10      %  refinement tolerance ||dx|| <= tol ||x||
  end

  properties (Access = private)
    h = uint64( 0 )         %  library handle (mnpbem_geom*)
  end

  methods
    function obj = bemretgpu( p, varargin )
      %  Initialize the GPU solver (geometry, refinement coefficients and
      %  closed-surface sum rule are computed once on the device).
      %  Usage :  obj = bemretgpu( p, op ),  obj = bemretgpu( p, enei, op )
      obj.p = p;
      op = struct;
      for i = 1 : numel( varargin )
        if isstruct( varargin{ i } ),  op = varargin{ i };  end
      end
      if isfield( op, 'precision' ),   obj.precision = op.precision;    end
      if isfield( op, 'refine_tol' ),  obj.refine_tol = op.refine_tol;  end
      %  concatenated vertices and faces of the compound, 0-based indices
      verts = [];  faces = [];  nfaces = zeros( 1, numel( p.p ), 'int64' );
      for i = 1 : numel( p.p )
        f = p.p{ i }.faces;
        f( isnan( f ) ) = 0;
        faces = [ faces; f + size( verts, 1 ) ];                 %#ok<AGROW>
        verts = [ verts; p.p{ i }.verts ];                       %#ok<AGROW>
        nfaces( i ) = size( f, 1 );
      end
      faces = int64( faces ) - 1;              %  triangles: 4th corner 0 - 1 = -1
      closed = zeros( 1, numel( p.p ), 'int32' );
      closed( [ p.closed{ : } ] ) = 1;
      q = p.p{ 1 }.quad;
      quad = struct( 'x', q.x, 'y', q.y, 'w', q.w, 'x3', q.x3, 'y3', q.y3, 'w3', q.w3,  ...
                     'x4', q.x4, 'y4', q.y4, 'w4', q.w4 );
      obj.h = mnpbem_gpu_mex( 'init', verts.', faces.', nfaces, int32( p.inout ).', closed, quad, op );
    end

    function delete( obj )
      %  Free the library handle and its device memory.
      if obj.h ~= 0,  mnpbem_gpu_mex( 'free', obj.h );  end
    end

    function sig = mldivide( obj, exc )
      %  sig = bem \ exc( p, enei ) (BEM/@bemret/mldivide.m): surface charges
      %  and currents for the external potentials of the excitation compstruct
      %  (phi1, phi1p, phi2, phi2p [n x npol], a1, a1p, a2, a2p [n x 3 x npol];
      %  missing fields are zero), as planewaveret or dipoleret return them.
      enei = exc.enei;
      eps = cellfun( @( e ) e( enei ), obj.p.eps );
      names = { 'phi1', 'phi1p', 'phi2', 'phi2p', 'a1', 'a1p', 'a2', 'a2p' };
      pot = cell( 1, 8 );
      for k = 1 : 8
        if isfield( exc, names{ k } ) && ~isempty( exc.( names{ k } ) )
          v = exc.( names{ k } );
          if k <= 4,  pot{ k } = complex( permute( v, [ 2, 1 ] ) );
          else,       pot{ k } = complex( permute( v, [ 3, 2, 1 ] ) );  end
        else
          pot{ k } = [];
        end
      end
      [ s1, s2, h1, h2 ] = mnpbem_gpu_mex( 'solve_pot', obj.h, enei, complex( eps( : ) ),  ...
                                           obj.precision, obj.refine_tol, pot{ : } );
      sig = compstruct( obj.p, enei, 'sig1', permute( s1, [ 2, 1 ] ),  ...
                                     'sig2', permute( s2, [ 2, 1 ] ),  ...
                                     'h1',   permute( h1, [ 3, 2, 1 ] ),  ...
                                     'h2',   permute( h2, [ 3, 2, 1 ] ) );
      obj.enei = enei;
    end

    function [ sig, ext, sca ] = solve( obj, pw, enei )
      %  One wavelength of a plane wave pw = planewaveret( pol, dir, op ): the
      %  excitation is evaluated on the device; returns sig and the cross
      %  sections the library computed from it (exc.ext / exc.sca of MNPBEM).
      %  One wavelength: compstruct sig plus the extinction and scattering
      %  cross sections the library computed from it.
      eps = cellfun( @( e ) e( enei ), obj.p.eps );
      [ ext, sca, s1, s2, h1, h2 ] = spectrum_( obj, pw, enei, eps( : ) );
      sig = compstruct( obj.p, enei, 'sig1', permute( s1, [ 2, 1 ] ),  ...
                                     'sig2', permute( s2, [ 2, 1 ] ),  ...
                                     'h1',   permute( h1, [ 3, 2, 1 ] ),  ...
                                     'h2',   permute( h2, [ 3, 2, 1 ] ) );
      ext = ext.';  sca = sca.';
      obj.enei = enei;
    end

    function [ ext, sca ] = spectrum( obj, pw, enei )
      %  A whole wavelength sweep in one library call: ext, sca [nenei x npol].
      eps = zeros( numel( obj.p.eps ), numel( enei ) );
      for k = 1 : numel( enei )
        eps( :, k ) = cellfun( @( e ) e( enei( k ) ), obj.p.eps );
      end
      [ ext, sca ] = spectrum_( obj, pw, enei, eps );
      ext = ext.';  sca = sca.';
    end

    function set_option( obj, key, value )
      %  Tuning option of the handle (lanes, lu_steps, gj_block, tc_stages, ...).
      mnpbem_gpu_mex( 'option', obj.h, key, value );
    end
  end

  methods (Access = private)
    function varargout = spectrum_( obj, pw, enei, eps )
      pinf = pw.spec.pinfty;
      [ varargout{ 1 : nargout } ] = mnpbem_gpu_mex( 'solve', obj.h, pw.pol.', pw.dir.', pw.medium,  ...
          pinf.nvec.', pinf.area( : ).', enei( : ).', complex( eps ), obj.precision, obj.refine_tol );
    end
  end
end
