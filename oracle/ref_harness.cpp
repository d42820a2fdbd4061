//==============================================================================
// ref_harness.cpp -- step-level harness around the REFERENCE CPU solver
// (test infrastructure: it generates the golden fixtures that pin the oracle).
//
// Built by oracle/Makefile.ref against the reference's own objects, compiled
// out of tree from the reference source.  It subclasses JSphCpuSingle (all its
// arrays and step methods are protected: JSphCpu.h:122-460,
// JSphCpuSingle.h:37-107), loads a case exactly as JSphCpuSingle::Run does
// (JSphCpuSingle.cpp:1144-1175), then runs the step piece by piece
// (ComputeStep_Sym, JSphCpuSingle.cpp:897-936) and dumps the solver arrays as
// raw little-endian files plus a key=value text file per stage.
//
//   ref_harness <casedir> <casename> <outdir> <nsteps_after_first> <threads>
//==============================================================================
#include <chrono>
#include "JSphCpuSingle.h"
#include "JSphCfgRun.h"
#include "JDsGaugeSystem.h"
#include "JDsGaugeItem.h"
#include "JDsMotion.h"
#include "JAppInfo.h"
#include "JLog2.h"
#include "JCellDivCpuSingle.h"
#include "JException.h"
#include "Functions.h"
#include "FunGeo3d.h"
#include "JMeshData.h"
#include <cfloat>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

JAppInfo AppInfo("DualSPHysics5","v5.4.355","08-04-2025");

namespace {

void WriteRaw(const std::string& file,const void* p,size_t bytes){
  FILE* f=fopen(file.c_str(),"wb");
  if(!f){ fprintf(stderr,"cannot write %s\n",file.c_str()); exit(2); }
  if(bytes)fwrite(p,1,bytes,f);
  fclose(f);
}

}

class OracleCpu : public JSphCpuSingle{
 public:
  std::string Out;
  std::vector<double> DtList;

  void Prepare(const std::string& appname,const JSphCfgRun* cfg,JLog2* log){
    // Same sequence as JSphCpuSingle::Run up to the main loop (JSphCpuSingle.cpp:1144-1175).
    AppName=appname; Log=log; CfgRun=cfg;
    Arrays_Cpu=new JArraysCpu(Log);
    Timersc->Config(cfg->SvTimers);
    LoadConfig(cfg);
    LoadCaseParticles();
    VisuConfig();
    ConfigDomain();
    ConfigRunMode();
    InitRunCpu();
    FreePartsInit();
    UpdateMaxValues();
    Part++;
    InterStep=INTERSTEP_SymPredictor;
  }

  void Meta(const std::string& tag,const std::string& extra=""){
    std::ofstream f((Out+"/"+tag+"_meta.txt").c_str());
    const StDivDataCpu dv=CellDivSingle->GetCellDivData();
    f.precision(17);
    f<<"np="<<Np<<"\nnpb="<<Npb<<"\nnpbok="<<NpbOk<<"\n";
    f<<"ncx="<<dv.nc.x<<"\nncy="<<dv.nc.y<<"\nncz="<<dv.nc.z<<"\nnsheet="<<dv.nc.w<<"\n";
    f<<"cellmin="<<dv.cellzero.x<<","<<dv.cellzero.y<<","<<dv.cellzero.z<<"\n";
    f<<"cellfluid="<<dv.cellfluid<<"\n";
    f<<"domcellcode="<<DomCellCode<<"\n";
    f<<"scell="<<Scell<<"\nkernelh="<<KernelH<<"\nkernelsize="<<KernelSize<<"\nkernelsize2="<<KernelSize2<<"\n";
    f<<"cs0="<<Cs0<<"\neta2="<<Eta2<<"\nddtkh="<<DDTkh<<"\nddtgz="<<DDTgz<<"\n";
    f<<"awen="<<KWend.awen<<"\nbwenh="<<KWend.bwenh<<"\n";
    f<<"cteb="<<CteB<<"\ngamma="<<Gamma<<"\nrhopzero="<<RhopZero<<"\nmassfluid="<<MassFluid<<"\nmassbound="<<MassBound<<"\n";
    f<<"dtini="<<DtIni<<"\ndtmin="<<DtMin<<"\ncflnumber="<<CFLnumber<<"\nmovlimit="<<MovLimit<<"\n";
    f<<"maprealposmin="<<MapRealPosMin.x<<","<<MapRealPosMin.y<<","<<MapRealPosMin.z<<"\n";
    f<<"maprealposmax="<<MapRealPosMax.x<<","<<MapRealPosMax.y<<","<<MapRealPosMax.z<<"\n";
    f<<"domposmin="<<DomPosMin.x<<","<<DomPosMin.y<<","<<DomPosMin.z<<"\n";
    f<<"mapcells="<<Map_Cells.x<<","<<Map_Cells.y<<","<<Map_Cells.z<<"\n";
    f<<"symplecticdtpre="<<SymplecticDtPre<<"\n";
    f<<"acemax="<<AceMax<<"\nvelmax="<<VelMax<<"\nviscdtmax="<<ViscDtMax<<"\n";
    f<<"timestep="<<TimeStep<<"\nnstep="<<Nstep<<"\n";
    f<<extra;
  }

  void DumpState(const std::string& tag){
    const std::string b=Out+"/"+tag+"_";
    WriteRaw(b+"idp.bin",Idp_c->cptr(),sizeof(unsigned)*Np);
    WriteRaw(b+"code.bin",Code_c->cptr(),sizeof(typecode)*Np);
    WriteRaw(b+"dcell.bin",Dcell_c->cptr(),sizeof(unsigned)*Np);
    WriteRaw(b+"pos.bin",Pos_c->cptr(),sizeof(tdouble3)*Np);
    WriteRaw(b+"velrho.bin",Velrho_c->cptr(),sizeof(tfloat4)*Np);
  }

  void DumpDivide(const std::string& tag){
    const StDivDataCpu dv=CellDivSingle->GetCellDivData();
    const unsigned nct=unsigned(dv.nc.w)*unsigned(dv.nc.z);
    const unsigned nctt=nct*2+6;
    WriteRaw(Out+"/"+tag+"_begincell.bin",dv.begincell,sizeof(unsigned)*nctt);
  }

  void DumpForces(const std::string& tag){
    const std::string b=Out+"/"+tag+"_";
    WriteRaw(b+"ace.bin",Ace_c->cptr(),sizeof(tfloat3)*Np);
    WriteRaw(b+"ar.bin",Ar_c->cptr(),sizeof(float)*Np);
    WriteRaw(b+"velrho.bin",Velrho_c->cptr(),sizeof(tfloat4)*Np);
    if(Shifting)WriteRaw(b+"shiftpos.bin",ShiftPosfs_c->cptr(),sizeof(tfloat4)*Np);
  }

  // Shifting displacements after RunShifting (JSphCpu.cpp:2084-2088).
  void ShiftAndDump(double dt,const std::string& tag){
    if(!Shifting)return;
    RunShifting(dt);
    WriteRaw(Out+"/"+tag+"_shiftpos.bin",ShiftPosfs_c->cptr(),sizeof(tfloat4)*Np);
  }

  // Motion data of every moving object for the interval just computed by
  // CalcMotion (JDsMotion::GetMotionData): "<time> <dt> <ref> <type>
  // <linmov 3> <linvel 3> <matmov 16>" lines in motion.txt.
  FILE* MotionOut=NULL;
  void DumpMotion(double dt){
    if(!CaseNmoving)return;
    if(!MotionOut)MotionOut=fopen((Out+"/motion.txt").c_str(),"w");
    for(unsigned ref=0;ref<DsMotion->GetNumObjects();ref++){
      const StMotionData& m=DsMotion->GetMotionData(ref);
      fprintf(MotionOut,"%.17g %.17g %u %d",TimeStep,dt,ref,int(m.type));
      const double* lm=&m.linmov.x; const double* lv=&m.linvel.x;
      for(int c=0;c<3;c++)fprintf(MotionOut," %.17g",lm[c]);
      for(int c=0;c<3;c++)fprintf(MotionOut," %.17g",lv[c]);
      const tmatrix4d& a=m.matmov;
      const double mm[16]={a.a11,a.a12,a.a13,a.a14,a.a21,a.a22,a.a23,a.a24,a.a31,a.a32,a.a33,a.a34,a.a41,a.a42,a.a43,a.a44};
      for(int c=0;c<16;c++)fprintf(MotionOut," %.17g",mm[c]);
      fprintf(MotionOut,"\n");
    }
    fflush(MotionOut);
  }

  // First step piece by piece (ComputeStep_Sym, JSphCpuSingle.cpp:897-936;
  // with moving boundaries, CalcMotion at its start and RunMotion before the
  // divide that ends it, as the Run loop does, JSphCpuSingle.cpp:1183-1196).
  void FirstStepDetailed(){
    Meta("s0");
    DumpState("s0"); DumpDivide("s0");
    const double dt=SymplecticDtPre;
    if(CaseNmoving){ CalcMotion(dt); DumpMotion(dt); }
    InterStep=INTERSTEP_SymPredictor;
    DemDtForce=dt*0.5f;
    MdbcBoundCorrection(InterStep);
    DumpState("s0mdbc");
    PreInteraction_Forces(InterStep);
    Interaction_Forces(InterStep);
    DumpForces("s0pred");
    const double dt_p=DtVariable(false);
    char tx[256]; sprintf(tx,"dt=%.17g\ndt_p=%.17g\n",dt,dt_p);
    Meta("s0pred",tx);
    ShiftAndDump(dt*.5,"s0predsh");
    ComputeSymplecticPre(dt);
    PosInteraction_Forces();
    DumpState("s0pre");
    InterStep=INTERSTEP_SymCorrector;
    DemDtForce=dt;
    RunCellDivide(true);
    Meta("s0div");
    DumpState("s0div"); DumpDivide("s0div");
    MdbcBoundCorrection(InterStep);
    PreInteraction_Forces(InterStep);
    Interaction_Forces(InterStep);
    DumpForces("s0cor");
    const double dt_c=DtVariable(true);
    sprintf(tx,"dt=%.17g\ndt_c=%.17g\n",dt,dt_c);
    Meta("s0cor",tx);
    ShiftAndDump(dt,"s0corsh");
    ComputeSymplecticCorr(dt);
    PosInteraction_Forces();
    DumpState("s0corr");
    SymplecticDtPre=std::min(dt_p,dt_c);
    if(CaseNmoving)RunMotion(dt);
    TimeStep+=dt; Nstep++;
    RunCellDivide(true);
    DtList.push_back(dt);
    Meta("s1");
    DumpState("s1"); DumpDivide("s1");
  }

  // First Verlet step piece by piece (ComputeStep_Ver, JSphCpuSingle.cpp:873-892;
  // with moving boundaries, CalcMotion after DtVariable and RunMotion after
  // the update, as the Run loop does, JSphCpuSingle.cpp:1191-1194).
  void FirstStepVerlet(){
    Meta("s0");
    DumpState("s0"); DumpDivide("s0");
    InterStep=INTERSTEP_Verlet;
    MdbcBoundCorrection(InterStep);
    DumpState("s0mdbc");
    PreInteraction_Forces(InterStep);
    Interaction_Forces(InterStep);
    DumpForces("s0pred");
    const double dt=DtVariable(true);
    if(CaseNmoving){ CalcMotion(dt); DumpMotion(dt); }
    char tx[256]; sprintf(tx,"dt=%.17g\ndt_p=%.17g\n",dt,dt);
    Meta("s0pred",tx);
    ShiftAndDump(dt,"s0predsh");
    ComputeVerlet(dt);
    PosInteraction_Forces();
    DumpState("s0pre");
    if(CaseNmoving)RunMotion(dt);
    TimeStep+=dt; Nstep++;
    RunCellDivide(true);
    DtList.push_back(dt);
    Meta("s1");
    DumpState("s1"); DumpDivide("s1");
  }

  bool IsSymplectic()const{ return(TStep==STEP_Symplectic); }

  void RunSteps(unsigned n){
    for(unsigned c=0;c<n;c++){
      const double stepdt=ComputeStep();
      if(CaseNmoving){ DumpMotion(stepdt); RunMotion(stepdt); }
      RunCellDivide(true);
      TimeStep+=stepdt; Nstep++;
      DtList.push_back(stepdt);
    }
    Meta("end");
    DumpState("end"); DumpDivide("end");
    WriteRaw(Out+"/end_dtlist.bin",DtList.data(),sizeof(double)*DtList.size());
  }

  // Gauges of the final state with the reference's own gauge classes
  // (JGaugeSystem::AddGauge*, JGaugeItem::CalculeCpu).  Input lines:
  //   vel  x y z
  //   swl  x0 y0 z0 x2 y2 z2 pointdp masslimit
  //   maxz x y z height distlimit
  //   mesh ptref(3) vec1(3) vec2(3) vec3(3) dis1 dis2 dis3 dispt1 dispt2 dispt3
  //        dirdat(3) kclimit kcdummy masslimit
  // Output: one line per gauge with the result (velocity / surface point /
  // zmax); a mesh gauge writes "mesh npt1 npt2 npt3", then one "pt vx vy vz
  // vdir rhop" line per point and one "zs zsurf" line per column.
  // Adds the gauges listed in f to the gauge system; returns their kinds.
  std::vector<std::string> ParseGauges(FILE* f){
    std::vector<std::string> kinds;
    char kind[16];
    unsigned ng=0;
    while(fscanf(f,"%15s",kind)==1){
      const std::string k=kind,name=std::string("g")+std::to_string(ng++);
      if(k=="vel"){
        double x,y,z; if(fscanf(f,"%lf %lf %lf",&x,&y,&z)!=3)break;
        GaugeSystem->AddGaugeVel(name,0,1e30,0,true,TDouble3(x,y,z));
      }
      else if(k=="swl"){
        double x0,y0,z0,x2,y2,z2,pdp; float ml;
        if(fscanf(f,"%lf %lf %lf %lf %lf %lf %lf %f",&x0,&y0,&z0,&x2,&y2,&z2,&pdp,&ml)!=8)break;
        GaugeSystem->AddGaugeSwl(name,0,1e30,0,true,TDouble3(x0,y0,z0),TDouble3(x2,y2,z2),pdp,ml);
      }
      else if(k=="maxz"){
        double x,y,z,hgt; float dl;
        if(fscanf(f,"%lf %lf %lf %lf %f",&x,&y,&z,&hgt,&dl)!=5)break;
        GaugeSystem->AddGaugeMaxZ(name,0,1e30,0,true,TDouble3(x,y,z),hgt,dl);
      }
      else if(k=="mesh"){
        double v[18]; float d[3],kcl,kcd,ml; bool ok=true;
        for(unsigned c=0;c<18 && ok;c++)ok=(fscanf(f,"%lf",v+c)==1);
        if(!ok || fscanf(f,"%f %f %f %f %f %f",d,d+1,d+2,&kcl,&kcd,&ml)!=6)break;
        jmsh::StMeshBasic mb;
        mb.ptref=TDouble3(v[0],v[1],v[2]); mb.vec1=TDouble3(v[3],v[4],v[5]);
        mb.vec2=TDouble3(v[6],v[7],v[8]); mb.vec3=TDouble3(v[9],v[10],v[11]);
        mb.dis1=v[12]; mb.dis2=v[13]; mb.dis3=v[14];
        mb.dispt1=v[15]; mb.dispt2=v[16]; mb.dispt3=v[17];
        mb.dirdat=fgeo::VecUnitary(TFloat3(d[0],d[1],d[2]));
        GaugeSystem->AddGaugeMesh(name,0,1e30,0,true,mb,"vel,veldir,rhop,zsurf",0,0,kcl,kcd,ml);
      }
      else break;
      kinds.push_back(k);
    }
    return(kinds);
  }

  // Computes every gauge on the current divided state with the reference's
  // JGaugeSystem::CalculeCpu and writes their results to o.
  void CalculeAndWriteGauges(FILE* o,const std::vector<std::string>& kinds){
    GaugeSystem->ConfigArraysCpu(Pos_c,Code_c,Idp_c,Velrho_c);
    GaugeSystem->CalculeCpu(TimeStep,DivData,NpbOk,Npb,Np,false);
    for(unsigned c=0;c<unsigned(kinds.size());c++){
      JGaugeItem* g=GaugeSystem->GetGauge(c);
      if(kinds[c]=="vel"){
        const tfloat3 v=((JGaugeVelocity*)g)->GetResult().vel;
        fprintf(o,"vel %.9g %.9g %.9g\n",v.x,v.y,v.z);
      }
      else if(kinds[c]=="swl"){
        const tfloat3 v=((JGaugeSwl*)g)->GetResult().posswl;
        fprintf(o,"swl %.9g %.9g %.9g\n",v.x,v.y,v.z);
      }
      else if(kinds[c]=="maxz"){
        fprintf(o,"maxz %.9g\n",((JGaugeMaxZ*)g)->GetResult().zmax);
      }
      else{
        JGaugeMesh* gm=(JGaugeMesh*)g;
        const jmsh::StMeshPts m=gm->GetMesh();
        jmsh::JMeshData* md=gm->GetResult().meshdat;
        const tfloat3* vel=md->GetVarFloat3("Vel");
        const float* vdir=md->GetVarFloat("VelDir");
        const float* rhop=md->GetVarFloat("Rhop");
        const float* zsurf=md->GetVarFloat("Zsurf");
        fprintf(o,"mesh %u %u %u\n",m.npt1,m.npt2,m.npt3);
        for(unsigned p=0;p<m.npt;p++)fprintf(o,"pt %.9g %.9g %.9g %.9g %.9g\n",vel[p].x,vel[p].y,vel[p].z,vdir[p],rhop[p]);
        for(unsigned p=0;p<m.npt1*m.npt2;p++)fprintf(o,"zs %.9g\n",zsurf[p]);
      }
    }
  }

  void RunGauges(const std::string& infile){
    FILE* f=fopen(infile.c_str(),"r");
    if(!f)return;
    const std::vector<std::string> kinds=ParseGauges(f);
    fclose(f);
    FILE* o=fopen((Out+"/gauges_out.txt").c_str(),"w");
    CalculeAndWriteGauges(o,kinds);
    fclose(o);
  }

  // Long run with samples (series.txt: "<nsteps> <every>", then gauge lines):
  // steps as the Run loop does (ComputeStep, then RunCellDivide,
  // JSphCpuSingle.cpp:1183-1196) and, at step 0 and every <every> steps,
  // writes "sample <nstep> <time> <np> <nfluid> <xfront>" (xfront: the largest
  // x of a fluid particle) followed by the gauges' results.
  void RunSeries(const std::string& infile){
    FILE* f=fopen(infile.c_str(),"r");
    if(!f)return;
    unsigned nsteps=0,every=1;
    if(fscanf(f,"%u %u",&nsteps,&every)!=2 || !every){ fclose(f); return; }
    const std::vector<std::string> kinds=ParseGauges(f);
    fclose(f);
    FILE* o=fopen((Out+"/series_out.txt").c_str(),"w");
    for(unsigned c=0;c<=nsteps;c++){
      if(c){
        const double stepdt=ComputeStep();
        RunCellDivide(true);
        TimeStep+=stepdt; Nstep++;
      }
      if(c%every==0){
        const tdouble3* pos=Pos_c->cptr();
        const typecode* code=Code_c->cptr();
        double xf=-DBL_MAX; unsigned nf=0;
        for(unsigned p=0;p<Np;p++)if(CODE_IsFluid(code[p])){ nf++; if(pos[p].x>xf)xf=pos[p].x; }
        fprintf(o,"sample %u %.17g %u %u %.17g\n",Nstep,TimeStep,Np,nf,xf);
        CalculeAndWriteGauges(o,kinds);
      }
    }
    fclose(o);
  }
  // Timing (timing.txt: "<nsteps>"): steps as the Run loop does, wall clock
  // around the steps only (the case is loaded and divided before); writes
  // "steps <n> seconds <t> np <np>" to timing_out.txt.
  void RunTiming(const std::string& infile){
    FILE* f=fopen(infile.c_str(),"r");
    if(!f)return;
    unsigned nsteps=0;
    if(fscanf(f,"%u",&nsteps)!=1){ fclose(f); return; }
    fclose(f);
    const auto t0=std::chrono::steady_clock::now();
    for(unsigned c=0;c<nsteps;c++){
      const double stepdt=ComputeStep();
      RunCellDivide(true);
      TimeStep+=stepdt; Nstep++;
    }
    const double sec=std::chrono::duration<double>(std::chrono::steady_clock::now()-t0).count();
    FILE* o=fopen((Out+"/timing_out.txt").c_str(),"w");
    fprintf(o,"steps %u seconds %.6f np %u\n",nsteps,sec,Np);
    fclose(o);
  }
};

int main(int argc,char** argv){
  if(argc<6){
    fprintf(stderr,"usage: %s <casedir> <casename> <outdir> <nsteps> <threads> [run options]\n",argv[0]);
    return 1;
  }
  const std::string casedir=argv[1],casename=argv[2],outdir=argv[3];
  const unsigned nsteps=unsigned(atoi(argv[4]));
  const std::string thr=std::string("-ompthreads:")+argv[5];
  AppInfo.ConfigRunPaths(argv[0]);
  JSphCfgRun cfg;
  cfg.SetFeatureList(JSph::GetFeatureList());
  std::string casepath=casedir+"/"+casename;
  // run options after <threads> (e.g. -cellmode:half) go to the reference's own parser
  std::vector<std::string> args={"ref_harness","-cpu",thr,"-sv:none","-svres:0"};
  for(int i=6;i<argc;i++)args.push_back(argv[i]);
  args.push_back(casepath);
  args.push_back(outdir);
  std::vector<char*> av;
  for(auto& s:args)av.push_back(const_cast<char*>(s.c_str()));
  int rc=1;
  try{
    cfg.LoadArgv(int(av.size()),av.data());
    AppInfo.ConfigOutput(cfg.CreateDirs,cfg.CsvSepComa,cfg.DirOut,cfg.DirDataOut);
    AppInfo.LogInit(AppInfo.GetDirOut()+"/Run.out");
    JLog2* log=AppInfo.LogPtr();
    OracleCpu sph;
    sph.Out=outdir;
    sph.Prepare(AppInfo.GetFullName(),&cfg,log);
    if(fun::FileExists(casedir+"/timing.txt"))sph.RunTiming(casedir+"/timing.txt");
    else if(fun::FileExists(casedir+"/series.txt"))sph.RunSeries(casedir+"/series.txt");
    else{
      if(sph.IsSymplectic())sph.FirstStepDetailed();
      else sph.FirstStepVerlet();
      sph.RunSteps(nsteps);
      sph.RunGauges(casedir+"/gauges.txt");
    }
    rc=0;
  }
  catch(const JException& e){ fprintf(stderr,"JException: %s\n",e.what()); }
  catch(const std::exception& e){ fprintf(stderr,"exception: %s\n",e.what()); }
  catch(const std::string& e){ fprintf(stderr,"exception: %s\n",e.c_str()); }
  catch(const char* e){ fprintf(stderr,"exception: %s\n",e); }
  return rc;
}
